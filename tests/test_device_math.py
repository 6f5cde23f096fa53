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
        assert np.array_equal(hlist[hptr[node_tile[link_node]] + lslot], P.llist.reshape(-1, 2)[:, 1])


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
