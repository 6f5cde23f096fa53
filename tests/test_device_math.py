"""The library's __host__ __device__ arithmetic and plan builder, compiled
for the host (tests/native/probe.cu), against the oracle."""
import ctypes as C
import math

import numpy as np
import pytest

import emulate
import native_probe as npb
from exfem import workloads
from exfem.abi import EXFEM_WAVE_P, EXFEM_WAVE_SV
from oracle import oracle
from util import per_receiver_rel, rel


def ku(mu, lam):
    k = np.array([(lam + 2 * mu) / 4, lam / 4, mu / 4, (lam + 3 * mu) / 12])
    return k


def test_state_layout_groups():
    """The FP32 state offsets (row_off / state_at): a node's 2R values are
    its own contiguous block in any grouping; lg = R is the plain layout
    (n*2 + d)*R + r; with lg = RPT the x then y values of each thread's RPT
    right-hand sides are adjacent, starting at n*2R + 2*r0, aligned for one
    vector of 2 RPT values."""
    L = npb.lib()
    for R in (1, 2, 4, 6, 8, 12, 16, 24, 64):
        for lg in {R} | {k for k in (1, 2, 4) if R % k == 0}:
            for n in (0, 1, 7, 123456789):
                offs = [L.probe_state_at(R, lg, n, d, r) for d in (0, 1) for r in range(R)]
                assert sorted(offs) == list(range(n * 2 * R, (n + 1) * 2 * R)), (R, lg)
                for r0 in range(0, R, lg):
                    grp = [L.probe_state_at(R, lg, n, d, r0 + j) for d in (0, 1) for j in range(lg)]
                    assert grp == list(range(n * 2 * R + 2 * r0, n * 2 * R + 2 * r0 + 2 * lg)), (R, lg, r0)
                    assert (n * 2 * R + 2 * r0) % (2 * lg) == 0
                if lg == R:
                    assert offs == [(n * 2 + d) * R + r for d in (0, 1) for r in range(R)]


def test_calck_rebuilt_from_six_values_is_bitwise():
    """The FP64 kernels rebuild calck's 8x8 matrix from six per-element values
    computed on the host; every entry must carry the formula's own bits, for
    the materials of the configs and for random (mu, lambda)."""
    L = npb.lib()
    rng = np.random.default_rng(3)
    cases = [(2000.0 * 1000.0 ** 2, 2000.0 * (2000.0 ** 2 - 2 * 1000.0 ** 2)),   # configs 0/1
             (1800.0 * 300.0 ** 2, 1800.0 * (700.0 ** 2 - 2 * 300.0 ** 2)),      # valley infill
             (1.0, -0.5), (3.0, 0.0)]
    cases += [(float(a), float(b)) for a, b in zip(rng.uniform(1e5, 1e10, 200), rng.uniform(-5e9, 1e10, 200))]
    for mu, lam in cases:
        assert L.probe_calck_check(mu, lam) == -1, (mu, lam)


def test_closed_form_q4_matches_calck():
    rng = np.random.default_rng(3)
    L = npb.lib()
    for mu, lam in ((2e9, 4e9), (1.0, 0.0), (0.0, 1.0), (3.3e8, 1.7e8)):
        K = oracle.calck(mu, lam)
        k = ku(mu, lam)
        for _ in range(5):
            u = rng.standard_normal(8)
            ux, uy = np.ascontiguousarray(u[0::2]), np.ascontiguousarray(u[1::2])
            fx, fy = np.zeros(4), np.zeros(4)
            L.probe_q4_ku(*k, npb.dp(ux), npb.dp(uy), npb.dp(fx), npb.dp(fy))
            f = np.empty(8)
            f[0::2], f[1::2] = fx, fy
            assert rel(f, K @ u) < 1e-14
            for c in range(4):
                a, b = np.zeros(1), np.zeros(1)
                L.probe_q4_ku_corner(*k, npb.dp(ux), npb.dp(uy), c, npb.dp(a), npb.dp(b))
                assert abs(a[0] - fx[c]) <= 1e-14 * np.abs(f).max() and abs(b[0] - fy[c]) <= 1e-14 * np.abs(f).max()
                # the folded form of the FP32 kernels: -w times the corner force
                for w in (1.0, 0.5):
                    L.probe_q4_corner_acc(*k, npb.dp(ux), npb.dp(uy), c, w, npb.dp(a), npb.dp(b))
                    tol = 1e-14 * np.abs(f).max()
                    assert abs(a[0] + w * fx[c]) <= tol and abs(b[0] + w * fy[c]) <= tol


@pytest.mark.parametrize("kind", [1, 2, 4, 5, 6])
def test_drm_forces_match_multdrm(kind):
    rng = np.random.default_rng(kind)
    mu, lam, mass = 2e9, 4e9, 1.2e5
    K = oracle.calck(mu, lam)
    M = oracle.calcsqm()
    masks = {2: [1, 1, 0, 0, 0, 0, 1, 1], 4: [0, 0, 1, 1, 1, 1, 0, 0], 1: [0, 0, 0, 0, 1, 1, 1, 1],
             6: [1, 1, 0, 0, 1, 1, 1, 1], 5: [0, 0, 1, 1, 1, 1, 1, 1]}
    e = np.array(masks[kind], np.uint8)
    u0, a0 = rng.standard_normal(8), rng.standard_normal(8) * 30
    want = oracle.multdrm(K, u0, e) + oracle.multdrm(M, a0, e) * mass
    p = np.zeros(8)
    npb.lib().probe_drm_forces(npb.dp(ku(mu, lam)), mass, kind, npb.dp(u0), npb.dp(a0), npb.dp(p))
    assert rel(p, want) < 1e-14


@pytest.mark.parametrize("kind,deg", [(EXFEM_WAVE_P, 0), (EXFEM_WAVE_P, 35), (EXFEM_WAVE_SV, 0), (EXFEM_WAVE_SV, 22)])
def test_device_planewave_matches_oracle(kind, deg):
    L = npb.lib()
    for t in (-0.4, -0.05, 0.0, 0.13, 0.5):
        for x1, x3 in ((0.0, 0.0), (-350.0, 120.0), (900.0, 1500.0)):
            want = oracle.planewave(kind, 1.3, 2000.0, 1000.0, math.radians(deg), 3.0, t, x1, x3)
            got = np.zeros(6)
            assert L.probe_planewave(kind, 1.3, 2000.0, 1000.0, math.radians(deg), 3.0, t, x1, x3, npb.dp(got)) == 0
            got = got.reshape(3, 2).T
            assert np.allclose(got, want, rtol=1e-14, atol=1e-14 * np.abs(want).max())
            d = np.zeros(2)
            L.probe_planewave_u(kind, 1.3, 2000.0, 1000.0, math.radians(deg), 3.0, t, x1, x3, npb.dp(d))
            assert np.allclose(d, want[:, 0], rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("kind,deg", [(EXFEM_WAVE_P, 40), (EXFEM_WAVE_SV, 20)])
def test_fp32_free_field_matches_fp64(kind, deg):
    L = npb.lib()
    for t in (-0.3, 0.0, 0.21, 1.7):
        for x1, x3 in ((0.0, 0.0), (-1900.0, 700.0), (2500.0, 1800.0)):
            want = oracle.planewave(kind, 1.0, 3000.0, 1500.0, math.radians(deg), 5.0, t, x1, x3)
            u, a = np.zeros(2, np.float32), np.zeros(2, np.float32)
            fp = C.POINTER(C.c_float)
            assert L.probe_planewave32(kind, 1.0, 3000.0, 1500.0, math.radians(deg), 5.0, t, x1, x3,
                                       u.ctypes.data_as(fp), a.ctypes.data_as(fp)) == 0
            assert np.allclose(u, want[:, 0], rtol=0, atol=2e-6 * max(1.0, np.abs(want[:, 0]).max()))
            assert np.allclose(a, want[:, 2], rtol=0, atol=2e-6 * np.abs(want[:, 2]).max() + 1e-3)


def test_device_wave_setup_rejects_unsupported_angles():
    L = npb.lib()
    out = np.zeros(6)
    assert L.probe_planewave(EXFEM_WAVE_SV, 1.0, 2000.0, 1000.0, math.radians(30.5), 2.0, 0, 0, 0, npb.dp(out)) == -4
    assert L.probe_planewave(EXFEM_WAVE_P, 1.0, 2000.0, 1000.0, math.radians(90.0), 2.0, 0, 0, 0, npb.dp(out)) == -4


def test_plan_mass_equals_oracle_mass_bitwise():
    m = workloads.build("canyon", scale=0.15, steps=5, refine_band=20)
    P = npb.PlanView(m)
    o = oracle.run(m, nsteps=0)
    assert np.array_equal(P.mfull_ref, o["mfull"])


def test_plan_gather_lists_cover_every_incidence():
    m = workloads.build("canyon", scale=0.2, steps=5)
    P = npb.PlanView(m)
    na, nh = int(P.scalars[0]), int(P.scalars[1])
    assert nh == m.problem.nhanging and na + nh == m.nnodes
    own = np.diff(P.ownptr)
    assert own.sum() == 4 * m.nelems and (own > 0).all()
    # every hanging node's terms appear at half weight in exactly its two anchors
    half = P.tlist[(P.tlist & 1) == 1]
    hang_terms = own[na:].sum()
    assert half.size == 2 * hang_terms
    # the hanging node of entry i is internal node n_active + i
    assert np.array_equal(P.hang.reshape(-1, 3)[:, 0], na + np.arange(nh))


@pytest.mark.parametrize("tn", [1, 16, 32, 100])
def test_tile_halo_slots_point_at_the_right_nodes(tn):
    m = workloads.build("canyon", scale=0.2, steps=5)
    P = npb.PlanView(m)
    na = int(P.scalars[0])
    hptr, hlist, tslot, nslot, lslot, hmax = P.tiles(tn)
    econn = P.econn.reshape(-1, 4)
    assert len(hptr) == (na + tn - 1) // tn + 1 and hmax == np.diff(hptr).max()
    node_tile = np.arange(na) // tn
    term_node = np.repeat(np.arange(na), np.diff(P.tptr))
    base = hptr[node_tile[term_node]]
    e = (P.tlist >> 1) >> 2
    assert np.array_equal(hlist[base[:, None] + tslot], econn[e])
    assert np.array_equal(hlist[hptr[node_tile] + nslot], np.arange(na))
    link_node = np.repeat(np.arange(na), np.diff(P.lptr))
    if link_node.size:
        assert np.array_equal(hlist[hptr[node_tile[link_node]] + lslot], P.llist.reshape(-1, 2)[:, 0])


def _u16(a):
    return np.asarray(a, np.int64) & 0xFFFF


@pytest.mark.parametrize("name,tn", [("canyon", 8), ("canyon", 16), ("valley", 16), ("valley", 32)])
def test_pipeline_copies_cover_the_halo_and_stay_in_their_stage(name, tn):
    """The copies k_pipe32's producer warp issues per tile, replayed on the
    host with its own arithmetic (lane i takes runs i and 32 + i, slots by a
    scan of the run lengths): the halo runs rebuild the sorted halo exactly,
    every copy lands inside its region of the stage, every address and size
    is a multiple of 16 bytes, and the byte total is the expect_tx count."""
    m = workloads.build(name, scale=0.1, steps=5)
    P = npb.PlanView(m)
    na, nn = int(P.scalars[0]), m.nnodes
    hptr, hlist, tslot, nslot, lslot, hmax = P.tiles(tn)
    hdr, runs, nrec, tpack, tmax = P.pipe_pack(tn)
    assert len(hdr) == len(hptr) - 1
    for R in (4, 64):
        tmev = (tmax + 1) & ~1
        off = [hmax * 8 * R]
        off += [off[0] + tn * 8 * R, off[0] + tn * 12 * R, off[0] + tn * 16 * R, off[0] + tn * 16 * R + tn * 32]
        off.append(off[4] + (tmev * 8 + 15) // 16 * 16)
        stage = (off[5] + tmax * 16 + 127) // 128 * 128
        region_end = [off[0], off[1], off[2], off[3], off[4], off[5], stage]
        for t in range(len(hdr)):
            hc, nt, toff, nr = hdr[t]
            assert hc == hptr[t + 1] - hptr[t] and nr <= 64
            r = runs[t]
            assert (r[nr:, 1] == 0).all() and (r[:nr, 1] > 0).all() and (r[:nr].sum(axis=1) <= nn).all()
            nodes = np.concatenate([np.arange(a, a + c) for a, c in r[:nr]])
            assert np.array_equal(nodes, hlist[hptr[t]:hptr[t + 1]])
            ca, cb = r[:32, 1], r[32:, 1]
            offa = np.cumsum(ca) - ca
            offb = ca.sum() + np.cumsum(cb) - cb
            cnt = min(tn, na - t * tn)
            ntev = (nt + 1) & ~1
            copies = []   # (region, dst offset, src byte offset in its array, bytes)
            for lane in range(32):
                for (first, c), o in ((r[lane], offa[lane]), (r[32 + lane], offb[lane])):
                    if c:
                        copies.append((0, o * 8 * R, first * 8 * R, c * 8 * R))
            n0 = t * tn
            copies += [(1, off[0], n0 * 8 * R, cnt * 8 * R), (2, off[1], n0 * 4 * R, cnt * 4 * R),
                       (3, off[2], n0 * 4 * R, cnt * 4 * R), (4, off[3], n0 * 32, cnt * 32)]
            if nt:
                copies += [(5, off[4], toff * 16, ntev * 8), (6, off[5], toff * 16 + ntev * 8, nt * 16)]
            total = 0
            for reg, dst, src, nb in copies:
                lo = 0 if reg == 0 else region_end[reg - 1]
                assert dst % 16 == 0 and src % 16 == 0 and nb % 16 == 0 and nb > 0
                assert lo <= dst and dst + nb <= region_end[reg]
                total += nb
            assert total == hc * 8 * R + cnt * (16 * R + 32) + ntev * 8 + nt * 16 < 2 ** 20
            assert toff * 4 + 2 * ntev + 4 * nt <= len(tpack)


@pytest.mark.parametrize("name,tn", [("canyon", 8), ("valley", 16)])
def test_pipeline_records_decode_to_the_mesh(name, tn):
    """The node and term records, decoded as k_pipe32's consumers decode
    them, give back each node's terms in gather order: corners through the
    halo slots, the corner the node occupies, the element coefficients times
    the term weight, the node's own slot, DRM and anchor-link ranges."""
    m = workloads.build(name, scale=0.1, steps=5)
    P = npb.PlanView(m)
    na = int(P.scalars[0])
    hptr, hlist, tslot, nslot, lslot, hmax = P.tiles(tn)
    hdr, runs, nrec, tpack, tmax = P.pipe_pack(tn)
    econn = P.econn.reshape(-1, 4)
    ecoef = np.asarray(P.ecoef32).reshape(-1, 4)
    tp = tpack.view(np.uint32)
    for n in range(na):
        t = n // tn
        hc, nt, toff, nr = hdr[t]
        ntev = (nt + 1) & ~1
        meta = nrec[n, 4:].view(np.uint32)
        tb, tc = int(meta[0] & 0xFFFF), int(meta[0] >> 16)
        assert tc == P.tptr[n + 1] - P.tptr[n] and tb == P.tptr[n] - P.tptr[t * tn]
        assert hlist[hptr[t] + int(meta[1])] == n
        assert int(meta[2] & 0xFFFFFF) == P.dptr[n] and int(meta[2] >> 24) == P.dptr[n + 1] - P.dptr[n]
        assert int(meta[3] & 0xFFFFFF) == P.lptr[n] and int(meta[3] >> 24) == P.lptr[n + 1] - P.lptr[n]
        for j in range(tc):
            q = P.tptr[n] + j
            ent = int(P.tlist[q])
            e, cor, w = (ent >> 1) >> 2, (ent >> 1) & 3, 0.5 if ent & 1 else 1.0
            x, y = tp[4 * toff + 2 * (tb + j)], tp[4 * toff + 2 * (tb + j) + 1]
            slots = [x & 0x3FFF, x >> 16, y & 0xFFFF, y >> 16]
            assert (x >> 14) & 3 == cor
            assert np.array_equal(hlist[hptr[t] + np.array(slots, np.int64)], econn[e])
            k = tpack[4 * toff + 2 * ntev + 4 * (tb + j):][:4].view(np.float32)
            assert np.array_equal(k, ecoef[e] * np.float32(w))


@pytest.mark.parametrize("name,scale,steps,kw", [("homogeneous_rectangle", 0.125, 250, {}),
                                                  ("canyon", 0.15, 500, {"refine_band": 20})])
def test_kernel_emulation_matches_oracle(name, scale, steps, kw):
    m = workloads.build(name, scale=scale, steps=steps, save_every=1, **kw)
    o = oracle.run(m, nthreads=8)
    e = emulate.emulate_fp64(m, steps)
    assert np.abs(o["seis"]).max() > 0.1
    assert per_receiver_rel(e["seis"], o["seis"]).max() < 1e-10


def test_fp32_increment_scheme_emulation_tracks_oracle():
    """The FP32 scheme (increment form, Kahan on u and D, bf16 compensations)
    emulated in float32 numpy: well inside the 1e-4 seismogram bar."""
    m = workloads.build("canyon", scale=0.15, steps=900, save_every=3, refine_band=20)
    o = oracle.run(m, rhs=4, nthreads=8)
    e = emulate.emulate_fp32(m, 900, rhs=4)
    assert per_receiver_rel(e["seis"], o["seis"]).max() < 1e-5


def test_tensor_core_tiles_cover_every_term():
    """build_mma_tiles (the tensor-core step's tiles): consecutive runs of at
    most 32 active nodes covering them all, at most 64 distinct elements per
    tile, and every gather term's index naming its own element in its tile's
    list."""
    m = workloads.build("valley_batched", scale=0.1, steps=4)
    P = npb.PlanView(m)
    nptr, eptr, elist, tj = P.mma_tiles(32, 64)
    na = int(P.scalars[0])
    assert nptr[0] == 0 and nptr[-1] == na and np.all(np.diff(nptr) >= 1) and np.all(np.diff(nptr) <= 32)
    assert np.all(np.diff(eptr) <= 64) and eptr[-1] == len(elist)
    tptr, tlist = P.tptr, P.tlist
    for t in range(len(nptr) - 1):
        els = elist[eptr[t]:eptr[t + 1]]
        assert len(set(els.tolist())) == len(els)
        q0, q1 = tptr[nptr[t]], tptr[nptr[t + 1]]
        assert np.array_equal(els[tj[q0:q1]], (tlist[q0:q1] >> 1) >> 2)
    # a tile closes early instead of exceeding its element budget
    nptr16, eptr16, _, _ = P.mma_tiles(32, 16)
    assert np.all(np.diff(eptr16) <= 16) and nptr16[-1] == na


def test_tensor_core_b_operand_is_the_q4_stiffness():
    """The tensor-core step's B operand is [Kmu; Klambda] = [calck(1, 0);
    calck(0, 1)] (formulation.f90:276-313; K is symmetric, so its rows are
    its columns), split into tf32 hi and lo parts: both parts have a 10-bit
    mantissa and hi + lo is the FP64 entry to 2^-21 relative."""
    b = np.zeros(256, np.float32)
    npb.lib().probe_mma_btile(b.ctypes.data_as(C.c_void_p))
    bits = b.view(np.uint32)
    assert np.all(bits & 0x1FFF == 0)

    def at(tile, n, k):   # the K-major core-matrix layout of the operand tile
        return tile[((n >> 3) * 256 + (k >> 2) * 128 + (n & 7) * 16 + (k & 3) * 4) // 4]

    hi, lo = b[:128], b[128:]
    for part, (mu, lam) in enumerate(((1.0, 0.0), (0.0, 1.0))):
        K = oracle.calck(mu, lam)
        for n in range(8):
            for k in range(8):
                got = float(at(hi, 8 * part + n, k)) + float(at(lo, 8 * part + n, k))
                assert abs(got - K[n, k]) <= 2.0 ** -21 * max(abs(K[n, k]), 1e-30), (part, n, k, got, K[n, k])


def test_node_slot_records_hold_each_nodes_first_terms():
    """build_node_slots (the direct gather's fixed-size node records): every
    active node's first four tlist entries in order, -1 past its last; a node
    is marked (invm -1) exactly when it has more than four terms, DRM terms,
    anchored hanging nodes, a dashpot or unequal x/y coefficients, and an
    unmarked node's invm is its 1/m_full bit for bit."""
    m = workloads.build("canyon", scale=0.2, steps=4)
    P = npb.PlanView(m)
    slot4, invm, marked, nc = P.node_slots()
    na = int(P.scalars[0])
    tptr, tlist, dptr, lptr = P.tptr, P.tlist, P.dptr, P.lptr
    cnt = np.diff(tptr[:na + 1])
    for j in range(4):
        has = cnt > j
        assert np.array_equal(slot4[has, j], tlist[tptr[:na][has] + j])
        assert np.all(slot4[~has, j] == -1)
    want = ((cnt > 4) | (np.diff(dptr[:na + 1]) > 0) | (np.diff(lptr[:na + 1]) > 0) | (nc[:, 2] != 0) |
            (nc[:, 3] != 0) | (nc[:, 0].view(np.uint32) != nc[:, 1].view(np.uint32)))
    assert np.array_equal(invm < 0, want) and marked == int(want.sum())
    assert np.all(invm[want] == -1.0)
    assert np.array_equal(invm[~want].view(np.uint32), nc[~want, 0].view(np.uint32))
    # the refined canyon has every kind of marked node, and most are unmarked
    assert (cnt > 4).any() and (np.diff(dptr[:na + 1]) > 0).any() and (np.diff(lptr[:na + 1]) > 0).any()
    assert (nc[:, 2] != 0).any() and marked < na // 4
