"""FP32 increment form with Kahan-compensated displacements, batched over
right-hand sides, against the FP64 oracle and the FP64 GPU form.

Tolerance: <= 1e-4 relative L2 per receiver seismogram (both components over
time); peak-amplitude error is checked at the same level."""
import math
import os

import numpy as np
import pytest

from exfem import decks, workloads
from exfem.abi import EXFEM_E_NAN, EXFEM_E_TIMEOUT, EXFEM_FP32_KAHAN, ExfemError
from exfem.gpu import Solver, estimate_bytes
from exfem.model import Model
from oracle import oracle
from util import peak_rel, per_receiver_rel

pytestmark = pytest.mark.gpu
TOL = 1e-4
NT = os.cpu_count() or 8


def run32(m, steps=None, **opts):
    with Solver(m, precision=EXFEM_FP32_KAHAN, **opts) as s:
        s.init_explicit()
        s.run(steps)
        s.sync()
        return s.seismograms(), [s.u(r) for r in range(s.nrhs)]


def test_rectangle_fp32_vs_oracle():
    m = workloads.build("homogeneous_rectangle", scale=0.25, steps=600)
    o = oracle.run(m, nthreads=NT)
    g, _ = run32(m)
    assert per_receiver_rel(g[0], o["seis"]).max() <= TOL
    assert peak_rel(g[0], o["seis"]).max() <= TOL


@pytest.mark.parametrize("variant", [0, 1])
def test_canyon_fp32_every_rhs_vs_oracle(variant):
    m = workloads.build("canyon", scale=0.15, steps=900, save_every=2, refine_band=20)
    g, _ = run32(m, variant=variant)
    for r in range(m.problem.nrhs):
        o = oracle.run(m, rhs=r, nthreads=NT)
        assert np.abs(o["seis"]).max() > 0.1
        assert per_receiver_rel(g[r], o["seis"]).max() <= TOL, r


@pytest.mark.parametrize("variant,rpt", [(0, 1), (0, 2), (0, 4), (1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4),
                                         (3, 4)])
def test_batched_valley_rhs_match_oracle_for_every_kernel_and_tile(variant, rpt):
    m = workloads.build("valley_batched", scale=0.1, steps=500, save_every=5)
    assert m.problem.nrhs == 64
    g, _ = run32(m, rhs_per_thread=rpt, block_threads=128 * rpt, variant=variant)
    for r in (0, 21, 40, 63):
        o = oracle.run(m, rhs=r, nthreads=NT)
        err = per_receiver_rel(g[r], o["seis"])
        assert err.max() <= TOL, (r, err.max())


def test_result_is_the_same_alone_and_in_the_batch():
    batch = workloads.build("valley_batched", scale=0.1, steps=300, save_every=3)
    gb, _ = run32(batch)
    waves = batch.waves()
    for r in (5, 37):
        w = waves[r]
        kind = "WAVEP" if w.kind == 1 else "WAVESV"
        alone = Model(decks.valley(scale=0.1, steps=300, rhs=[(kind, w.angle, w.amp, w.freq)]), nsteps=300,
                      io_interval=3)
        assert abs(alone.waves()[0].t0 - w.t0) < 1e-12
        ga, _ = run32(alone)
        assert per_receiver_rel(ga[0], gb[r]).max() <= 1e-6


def test_fp32_vs_fp64_gpu_on_full_canyon():
    """Full-size canyon (~1.9e5 elements, hanging nodes), 4000 steps (2.5 s,
    past every wave's arrival): the FP32 form against the FP64 form, per
    receiver and right-hand side."""
    m = workloads.build("canyon", steps=4000)
    g32, _ = run32(m)
    with Solver(m) as s:
        s.init_explicit()
        s.run()
        s.sync()
        g64 = s.seismograms()
    for r in range(m.problem.nrhs):
        assert np.abs(g64[r]).max() > 0.1
        assert per_receiver_rel(g32[r], g64[r]).max() <= TOL, r


def test_fp32_vs_fp64_gpu_on_full_valley_full_length():
    """The valley at full size and length (1.5M elements, four quadtree
    levels, heterogeneous infill, 20,000 steps): the FP32 form against the
    plain FP64 form, relative L2 and peak amplitude per receiver (measured:
    6.5e-7 and 4.0e-7)."""
    m = workloads.build("valley", steps=20000)
    assert m.nelems > 1_400_000 and m.problem.nhanging > 0
    g32, _ = run32(m)
    with Solver(m) as s:
        s.init_explicit()
        s.run()
        s.sync()
        g64 = s.seismograms()
    assert np.abs(g64[0]).max() > 0.1
    assert per_receiver_rel(g32[0], g64[0]).max() <= TOL
    assert peak_rel(g32[0], g64[0]).max() <= TOL


def test_diverging_run_is_reported():
    """dt five times over the stability limit: the watchdog turns the blow-up
    into EXFEM_E_NAN at sync instead of silent garbage."""
    d = decks.homogeneous_rectangle(scale=0.125, steps=400, save_every=10).replace("CONTROL:\n10.0 2.0",
                                                                                    "CONTROL:\n10.0 0.4")
    m = Model(d)   # the deck's TIME now gives 80 steps of the larger dt
    with Solver(m, precision=EXFEM_FP32_KAHAN) as s:
        s.init_explicit()
        s.run()
        with pytest.raises(ExfemError) as e:
            s.sync()
        assert e.value.code == EXFEM_E_NAN


def test_autotuner_picks_a_working_shape():
    """exfem_gpu_autotune (through exfem.autotune) writes a shape that runs
    and gives the same results as the default shape; a second call on the
    same mesh comes from the library's cache."""
    import time

    from exfem import autotune
    m = workloads.build("valley_batched", scale=0.1, steps=40)
    choice = autotune.tune(m, steps=8)
    assert choice["rhs_per_thread"] in (1, 2, 4) and choice["block_threads"] in (128, 256, 512)
    assert choice["variant"] in (0, 1, 2, 3, 4, 5) and choice["ms_per_step"] > 0
    t0 = time.perf_counter()
    again = autotune.tune(m, steps=8)
    assert time.perf_counter() - t0 < 0.05 and again == choice
    a, ua = run32(m, variant=0)
    b, ub = run32(m, variant=choice["variant"], block_threads=choice["block_threads"],
                  rhs_per_thread=choice["rhs_per_thread"])
    assert np.array_equal(a, b)


def test_tiled_and_direct_kernels_agree():
    """The tiled kernel sums the same terms in the same order as the direct
    gather, from shared memory: bit for bit the same state."""
    m = workloads.build("canyon", scale=0.2, steps=300, save_every=3)
    a, ua = run32(m, variant=0)
    b, ub = run32(m, variant=1)
    assert np.array_equal(a, b)
    for r in range(m.problem.nrhs):
        assert np.array_equal(ua[r], ub[r]), r


def test_padded_rhs_match_unpadded():
    """The FP32 form pads odd right-hand-side counts with zero-amplitude waves
    (9 -> 10, 13 -> 16): the caller's seismograms and state are bit for bit
    those of the unpadded run, every output covers only the caller's
    right-hand sides, and the footprint estimate still bounds the context."""
    for waves in (EIGHT_WAVES + [("WAVEP", 10.0)], EIGHT_WAVES + EIGHT_WAVES[:5]):
        m = workloads.build("canyon", scale=0.2, steps=60, save_every=2, waves=waves)
        R = m.problem.nrhs
        assert R in (9, 13) and m.problem.nhanging > 0
        a, ua = run32(m, pad_rhs=1)
        b, ub = run32(m)
        assert a.shape[0] == b.shape[0] == R
        assert np.array_equal(a, b)
        for r in range(R):
            assert np.array_equal(ua[r], ub[r]), r
        with Solver(m, precision=EXFEM_FP32_KAHAN) as s:
            s.init_explicit()
            assert estimate_bytes(m, precision=EXFEM_FP32_KAHAN) >= s.device_bytes
            with pytest.raises(ExfemError):
                s.u(R)
        o = oracle.run(m, rhs=R - 1, nthreads=NT)
        assert per_receiver_rel(b[R - 1], o["seis"]).max() <= TOL


@pytest.mark.parametrize("nrhs", [96, 128])
def test_many_rhs_match_oracle_and_fewer_rhs(nrhs):
    """Batches wider than the 64-RHS valley: at four RHS per thread a node
    takes 24 threads (R = 96, not a power of two) or 32 (R = 128, a whole
    warp).  The first and last RHS match the oracle, and every RHS is bit for
    bit the same as in a 16-RHS batch of the same waves."""
    waves = [("WAVEP" if i % 2 == 0 else "WAVESV", (3.0 + 0.4 * i) % 25.0) for i in range(nrhs)]
    m = workloads.build("canyon", scale=0.15, steps=120, save_every=2, waves=waves)
    assert m.problem.nrhs == nrhs
    g, u = run32(m)
    for r in (0, nrhs - 1):
        o = oracle.run(m, rhs=r, nthreads=NT)
        assert per_receiver_rel(g[r], o["seis"]).max() <= TOL, r
    m16 = workloads.build("canyon", scale=0.15, steps=120, save_every=2, waves=waves[nrhs - 16:])
    g16, u16 = run32(m16)
    assert np.array_equal(g[nrhs - 16:], g16)
    for k in range(16):
        assert np.array_equal(u[nrhs - 16 + k], u16[k])


def test_get_u_copies_one_rhs():
    """exfem_gpu_get_u gathers the requested right-hand side on the device:
    2 * nnodes doubles cross to the host, not the batched state (FP32 and
    FP64 contexts)."""
    m = workloads.build("valley_batched", scale=0.08, steps=20)
    assert m.problem.nrhs == 64
    for prec in (EXFEM_FP32_KAHAN, 0):
        with Solver(m, precision=prec) as s:
            s.init_explicit()
            s.run(6)
            s.sync()
            _, d0 = s.copy_bytes()
            u = s.u(37)
            _, d1 = s.copy_bytes()
            assert u.size == 2 * m.nnodes
            assert d1 - d0 == 2 * m.nnodes * 8
            assert np.isfinite(u).all()


@pytest.mark.parametrize("rpt", [4, 2, 1])
def test_32_and_64_bit_indices_agree(rpt):
    """k_step32's 32-bit index form (shift and mask thread split) and its
    64-bit form compute the same terms in the same order: the same state bit
    for bit, on a batched valley with hanging nodes and a DRM layer; and a
    thread count per node that is not a power of two (12 RHS) takes the
    division path."""
    m = workloads.build("valley_batched", scale=0.1, steps=60, save_every=2)
    assert m.problem.nhanging > 0 and m.problem.nseismic > 0 and m.problem.nrhs == 64
    a, ua = run32(m, variant=0, rhs_per_thread=rpt)
    b, ub = run32(m, variant=0, rhs_per_thread=rpt, index_bits=64)
    assert np.array_equal(a, b)
    for r in range(m.problem.nrhs):
        assert np.array_equal(ua[r], ub[r]), r
    m12 = workloads.build("canyon", scale=0.2, steps=60, save_every=2, waves=EIGHT_WAVES + EIGHT_WAVES[:4])
    assert m12.problem.nrhs == 12
    a, ua = run32(m12, variant=0, rhs_per_thread=rpt)
    b, ub = run32(m12, variant=0, rhs_per_thread=rpt, index_bits=64)
    assert np.array_equal(a, b)
    for r in range(m12.problem.nrhs):
        assert np.array_equal(ua[r], ub[r]), r


def test_paired_rows_match_split_rows():
    """With one thread per node (one, two or four RHS at as many per thread)
    k_step32 moves a node's x and y rows as one 8-, 16- or 32-byte vector;
    the terms and their order are those of the split form.  On a valley with
    hanging nodes and a DRM layer: two RHS at one per thread (split rows) and
    at two (paired); four RHS at one and two per thread (split) and at four
    (paired); three RHS (padded to four, paired) against the first three of
    the four.  The same seismograms and state bit for bit; each of the two
    RHS alone (paired) as in the batch (its wave's delay is recomputed alone,
    hence 1e-6) and within the tolerance of the oracle."""
    waves = [("WAVESV", 0.0, 1.0, 5.0), ("WAVEP", math.radians(15.0), 1.0, 5.0),
             ("WAVESV", math.radians(10.0), 0.7, 3.0), ("WAVEP", math.radians(40.0), 1.2, 4.0)]
    m = Model(decks.valley(scale=0.1, steps=2000, rhs=waves[:2]), nsteps=2000, io_interval=4)
    assert m.problem.nhanging > 0 and m.problem.nseismic > 0 and m.problem.nrhs == 2
    a, ua = run32(m, variant=0, rhs_per_thread=1)
    b, ub = run32(m, variant=0, rhs_per_thread=2)
    assert np.array_equal(a, b)
    for r in range(2):
        assert np.array_equal(ua[r], ub[r]), r
    m4 = Model(decks.valley(scale=0.1, steps=600, rhs=waves), nsteps=600, io_interval=4)
    runs = [run32(m4, variant=0, rhs_per_thread=rpt) for rpt in (1, 2, 4)]
    for g, u in runs[1:]:
        assert np.array_equal(g, runs[0][0])
        for r in range(4):
            assert np.array_equal(u[r], runs[0][1][r]), r
    m3 = Model(decks.valley(scale=0.1, steps=600, rhs=waves[:3]), nsteps=600, io_interval=4)
    g3, u3 = run32(m3, variant=0)
    assert g3.shape[0] == 3 and np.array_equal(g3, runs[0][0][:3])
    for r in range(3):
        assert np.array_equal(u3[r], runs[0][1][r]), r
    for r in range(2):
        alone = Model(decks.valley(scale=0.1, steps=2000, rhs=[waves[r]]), nsteps=2000, io_interval=4)
        c, _ = run32(alone, variant=0)
        assert per_receiver_rel(c[0], a[r]).max() <= 1e-6, r
        o = oracle.run(alone, nthreads=NT)
        assert np.abs(o["seis"]).max() > 0.1
        assert per_receiver_rel(c[0], o["seis"]).max() <= TOL, r


def test_grouped_layouts_agree():
    """With several threads per node the direct gather groups each node's
    state by the thread's RHS (x then y values of one, two or four RHS side
    by side); the tiled kernel reads the plain layout.  Twelve RHS on a
    valley with hanging nodes, a DRM layer and receivers, at one, two and
    four RHS per thread and tiled: the same seismograms, state (get_u) and
    sampled field (sample_points) of every RHS bit for bit, and the
    oracle's seismograms within the tolerance."""
    waves = [("WAVEP" if i % 2 == 0 else "WAVESV", math.radians(2.0 * i), 1.0, 5.0) for i in range(12)]
    m = Model(decks.valley(scale=0.1, steps=1500, rhs=waves), nsteps=1500, io_interval=5)
    assert m.problem.nhanging > 0 and m.problem.nseismic > 0 and m.problem.nrhs == 12
    xy = m.nodes().reshape(-1, 2)
    grid = m.grid(0.0, xy[:, 0].max(), 0.0, xy[:, 1].max(), 40.0)
    assert grid["nfound"] > 0
    runs = []
    for opts in (dict(rhs_per_thread=1), dict(rhs_per_thread=2), dict(rhs_per_thread=4), dict(variant=1)):
        with Solver(m, precision=EXFEM_FP32_KAHAN, **opts) as s:
            s.init_explicit()
            s.run()
            s.sync()
            runs.append((s.seismograms(), [s.u(r) for r in range(12)],
                         [s.sample_points(grid["points"], grid["elem"], rhs=r) for r in range(12)]))
    assert np.abs(runs[0][2][11]).max() > 0
    for g, u, f in runs[1:]:
        assert np.array_equal(g, runs[0][0])
        for r in range(12):
            assert np.array_equal(u[r], runs[0][1][r]), r
            assert np.array_equal(f[r], runs[0][2][r]), r
    for r in (0, 11):
        o = oracle.run(m, rhs=r, nthreads=NT)
        assert np.abs(o["seis"]).max() > 0.1
        assert per_receiver_rel(runs[0][0][r], o["seis"]).max() <= TOL, r


EIGHT_WAVES = [("WAVEP", 0.0), ("WAVEP", 20.0), ("WAVEP", 40.0), ("WAVEP", 60.0),
               ("WAVESV", 0.0), ("WAVESV", 10.0), ("WAVESV", 20.0), ("WAVESV", 25.0)]


@pytest.mark.parametrize("block,rpt", [(256, 4), (128, 2), (512, 4)])
def test_pipelined_kernel_runs_and_matches_the_direct_gather(block, rpt):
    """Variant 2 (bulk-copy pipeline) on a refined canyon with 8 waves:
    k_pipe32 is what runs; it sums the same terms in the same order as the
    direct gather (weights folded into the coefficients by a power of two),
    so seismograms and final state are bit for bit the same; and both match
    the oracle."""
    m = workloads.build("canyon", scale=0.2, steps=300, save_every=3, waves=EIGHT_WAVES)
    assert m.problem.nhanging > 0 and m.problem.nrhs == 8
    with Solver(m, precision=EXFEM_FP32_KAHAN, variant=2, block_threads=block, rhs_per_thread=rpt) as s:
        s.init_explicit()
        names = s.kernel_times(4)
        assert "k_pipe32" in names and "k_step32" not in names, names
    a, ua = run32(m, variant=0)
    b, ub = run32(m, variant=2, block_threads=block, rhs_per_thread=rpt)
    assert np.array_equal(a, b)
    for r in range(m.problem.nrhs):
        assert np.array_equal(ua[r], ub[r]), r
    for r in (0, 5):
        o = oracle.run(m, rhs=r, nthreads=NT)
        assert per_receiver_rel(b[r], o["seis"]).max() <= TOL, r


def test_pipelined_variant_falls_back_when_rows_are_not_16_bytes():
    """6 right-hand sides give 24-byte rows: variant 2 runs the direct gather."""
    m = workloads.build("canyon", scale=0.15, steps=40, save_every=2)
    assert m.problem.nrhs % 4 != 0
    with Solver(m, precision=EXFEM_FP32_KAHAN, variant=2) as s:
        s.init_explicit()
        names = s.kernel_times(4)
    assert "k_step32" in names and "k_pipe32" not in names


def test_bounded_wait_runs_out_and_reports_a_status():
    """Variant 2's mbarrier waits are bounded (exfem_opts.wait_cycles).  With
    a bound of one cycle the consumers' first wait runs out before the bulk
    copies land: the kernel sets the watchdog flag, the producer waits (with
    the default bound) for the copies it issued, and the block returns.
    exfem_gpu_sync reports EXFEM_E_TIMEOUT; the device stays usable, and a
    context with the default bound on the same device runs and matches the
    direct gather bit for bit."""
    m = workloads.build("canyon", scale=0.15, steps=40, save_every=2, waves=EIGHT_WAVES)
    assert m.problem.nrhs == 8
    with Solver(m, precision=EXFEM_FP32_KAHAN, variant=2, wait_cycles=1) as s:
        s.init_explicit()
        names = s.kernel_times(2)
        assert "k_pipe32" in names, names
        with pytest.raises(ExfemError) as e:
            s.sync()
        assert e.value.code == EXFEM_E_TIMEOUT
        assert b"timed out" in s.lib.exfem_gpu_last_error(s.h)
    a, ua = run32(m, variant=0)
    b, ub = run32(m, variant=2)
    assert np.array_equal(a, b)
    # the tensor-core step's wait for its MMAs is bounded the same way: it
    # gives up, flags, still waits (with the default bound) for the MMAs
    # before it frees their TMEM, and returns
    m16 = workloads.build("canyon", scale=0.15, steps=40, save_every=2, waves=EIGHT_WAVES + EIGHT_WAVES)
    with Solver(m16, precision=EXFEM_FP32_KAHAN, variant=3, wait_cycles=1) as s:
        s.init_explicit()
        names = s.kernel_times(2)
        assert "k_mma32" in names, names
        with pytest.raises(ExfemError) as e:
            s.sync()
        assert e.value.code == EXFEM_E_TIMEOUT
    c, _ = run32(m16, variant=3)
    d, _ = run32(m16, variant=0)
    for r in range(16):
        assert per_receiver_rel(c[r], d[r]).max() <= TOL, r


@pytest.mark.parametrize("nrhs_waves", [1, 8, 12])
def test_in_context_tuning_keeps_results(nrhs_waves):
    """exfem_opts.tune times the direct gather's shapes on the context itself
    before the state is set up; whatever it picks, the run gives the same
    seismograms and state as the built-in shape, bit for bit."""
    waves = (EIGHT_WAVES + EIGHT_WAVES)[:nrhs_waves]
    m = workloads.build("canyon", scale=0.2, steps=60, save_every=2, waves=waves)
    a, ua = run32(m)
    b, ub = run32(m, tune=1)
    assert np.array_equal(a, b)
    for r in range(m.problem.nrhs):
        assert np.array_equal(ua[r], ub[r]), r


def test_tensor_core_step_runs_and_matches_the_direct_gather():
    """Variant 3: the element products on the tensor cores (k_mma32, tcgen05
    kind::tf32 in 3xTF32) are what runs; on the 64-RHS valley and on a
    16-RHS refined canyon (hanging nodes, DRM layer) every RHS stays within
    the FP32 tolerance of the direct gather, and the canyon's RHS match the
    oracle.  With 8 RHS (not a multiple of 16) the direct gather runs."""
    mv = workloads.build("valley_batched", scale=0.1, steps=40, save_every=2)
    with Solver(mv, precision=EXFEM_FP32_KAHAN, variant=3) as s:
        s.init_explicit()
        names = s.kernel_times(4)
    assert "k_mma32" in names and "k_step32" not in names, names
    a, _ = run32(mv, variant=0)
    b, _ = run32(mv, variant=3)
    for r in range(mv.problem.nrhs):
        assert per_receiver_rel(b[r], a[r]).max() <= TOL, r
    mc = workloads.build("canyon", scale=0.2, steps=300, save_every=3, waves=EIGHT_WAVES + EIGHT_WAVES)
    assert mc.problem.nrhs == 16 and mc.problem.nhanging > 0
    a, _ = run32(mc, variant=0)
    b, _ = run32(mc, variant=3)
    for r in range(16):
        assert per_receiver_rel(b[r], a[r]).max() <= TOL, r
    for r in (0, 13):
        o = oracle.run(mc, rhs=r, nthreads=NT)
        assert per_receiver_rel(b[r], o["seis"]).max() <= TOL, r
    m8 = workloads.build("canyon", scale=0.15, steps=20, waves=EIGHT_WAVES)
    with Solver(m8, precision=EXFEM_FP32_KAHAN, variant=3) as s:
        s.init_explicit()
        names = s.kernel_times(2)
    assert "k_step32" in names and "k_mma32" not in names, names


@pytest.mark.parametrize("use_graph", [1, 0])
def test_side_stream_drm_forces_match_the_inline_pass(use_graph):
    """exfem_opts.drm_inline = 0 (the default) computes the next step's DRM
    forces on a second stream while the step runs, into the other of two
    force slots; = 1 computes them inside the hanging/receiver pass.  Both
    evaluate the same forces for the same steps: seismograms and state are
    the same bit for bit, with graph replays mixed with single steps (the
    host's joins before replays and at the end of each run) and without
    graphs, on a refined canyon with 8 RHS and on the 64-RHS valley."""
    for m in (workloads.build("canyon", scale=0.2, steps=130, save_every=1, waves=EIGHT_WAVES),
              workloads.build("valley_batched", scale=0.08, steps=130, save_every=2)):
        runs = []
        for inline in (1, 0):
            with Solver(m, precision=EXFEM_FP32_KAHAN, drm_inline=inline, use_graph=use_graph) as s:
                s.init_explicit()
                for n in (1, 17, 40, 72):
                    s.run(n)
                s.sync()
                runs.append((s.seismograms(), [s.u(r) for r in range(s.nrhs)]))
        assert np.array_equal(runs[0][0], runs[1][0])
        for r in range(m.problem.nrhs):
            assert np.array_equal(runs[0][1][r], runs[1][1][r]), r


def test_persistent_step_matches_the_direct_gather():
    """Variant 4 runs the direct gather as a persistent grid (k_step32p: the
    blocks that fit at once stride over the tiles); it computes the same
    terms in the same order, so results are bit for bit those of variant 0."""
    for m in (workloads.build("canyon", scale=0.2, steps=80, save_every=2, waves=EIGHT_WAVES),
              workloads.build("valley_batched", scale=0.08, steps=80, save_every=2)):
        with Solver(m, precision=EXFEM_FP32_KAHAN, variant=4) as s:
            s.init_explicit()
            names = s.kernel_times(2)
        assert "k_step32p" in names and "k_step32" not in names, names
        a, ua = run32(m, variant=0)
        b, ub = run32(m, variant=4)
        assert np.array_equal(a, b)
        for r in range(m.problem.nrhs):
            assert np.array_equal(ua[r], ub[r]), r


SIXTEEN_WAVES = EIGHT_WAVES + [("WAVEP", 10.0), ("WAVEP", 30.0), ("WAVEP", 50.0), ("WAVEP", 70.0),
                               ("WAVESV", 5.0), ("WAVESV", 15.0), ("WAVESV", 22.0), ("WAVESV", 28.0)]


@pytest.mark.parametrize("nwaves,rpt", [(1, 0), (2, 0), (4, 0), (6, 0), (6, 1), (8, 2), (8, 4), (16, 0), (16, 2)])
def test_node_slot_records_match_the_list_form(nwaves, rpt):
    """The direct gather reads a common node's first four terms and 1/m_full
    from its fixed-size slot record (variant 0) and a marked node's DRM terms,
    extra terms, dashpot and anchors from the lists; variant 5 reads every
    node through the lists.  Same terms in the same order: bit-identical
    seismograms and final states, on a refined canyon (hanging nodes, anchors,
    DRM layer, dashpots) at every kernel shape (the slot form's term corners
    from econn up to 12 RHS, copies from 14, the list form's copies from 6;
    paired and split rows; 1, 2, 4 RHS per thread).  The records are used
    from 50,000 active nodes: this canyon has 59,682."""
    m = workloads.build("canyon", scale=0.55, steps=80, save_every=2, waves=SIXTEEN_WAVES[:nwaves])
    assert m.nnodes > 55000
    kw = dict(rhs_per_thread=rpt) if rpt else {}
    a, ua = run32(m, variant=0, **kw)
    b, ub = run32(m, variant=5, **kw)
    assert np.abs(a).max() > 0
    assert np.array_equal(a, b)
    for r in range(m.problem.nrhs):
        assert np.array_equal(ua[r], ub[r]), r


def test_node_slot_records_on_the_batched_valley_and_persistent_grid():
    """The 64-RHS valley (plain layout, term corner copies) and the persistent
    grid (variant 4, which also reads the slot records) against the list form."""
    m = workloads.build("valley_batched", scale=0.2, steps=60, save_every=2)
    assert m.nnodes > 55000
    a, ua = run32(m, variant=5)
    for v in (0, 4):
        b, ub = run32(m, variant=v)
        assert np.array_equal(a, b), v
        for r in range(0, m.problem.nrhs, 9):
            assert np.array_equal(ua[r], ub[r]), (v, r)


@pytest.mark.parametrize("use_graph", [1, 0])
def test_programmatic_dependent_launch_keeps_results(use_graph):
    """The direct gather's step kernel launches as a programmatic dependent of
    the hanging/receiver pass before it (exfem_opts.serial_launch = 0, the
    default): its blocks may start while that pass runs and wait for it before
    touching the state.  Bit-identical to serial launches, with graph replay
    and without, with the DRM forces inline and on the second stream, in the
    slot and list forms and the persistent grid."""
    canyon = workloads.build("canyon", scale=0.55, steps=70, save_every=2, waves=EIGHT_WAVES[:2])
    # a small mesh whose step is shorter than the next step's DRM pass on
    # the second stream: the forces are still being computed when the hanging
    # pass could start
    rect = workloads.build("homogeneous_rectangle", steps=120, save_every=1)
    for m, kws in ((canyon, (dict(), dict(drm_inline=1), dict(variant=5), dict(variant=4))), (rect, (dict(),))):
        for kw in kws:
            a, ua = run32(m, use_graph=use_graph, serial_launch=1, **kw)
            b, ub = run32(m, use_graph=use_graph, **kw)
            assert np.array_equal(a, b), kw
            for r in range(m.problem.nrhs):
                assert np.array_equal(ua[r], ub[r]), (kw, r)
