"""Plain FP64 form on the GPU against the CPU oracle, through the C ABI.

Tolerance: <= 1e-12 relative L2 per receiver seismogram (both components over
time) — the bar for the plain FP64 form.  The default kernels keep the
oracle's operation order, so in practice the gap is the exp() of the free
field (CUDA vs host libm)."""
import math
import os

import numpy as np
import pytest

from exfem import decks, workloads
from exfem.abi import (EXFEM_E_ARG, EXFEM_E_STATE, EXFEM_E_UNSUPPORTED, EXFEM_VARIANT_CLOSED_FORM, ExfemError)
from exfem.gpu import Solver
from exfem.model import Model
from oracle import oracle
from util import fp64_rel, per_receiver_rel, rel

pytestmark = pytest.mark.gpu
TOL = 1e-12
NT = os.cpu_count() or 8


def gpu_run(m, steps=None, **opts):
    with Solver(m, **opts) as s:
        mf = s.init_explicit()
        s.run(steps)
        s.sync()
        seis = s.seismograms()
        us = [s.u(r) for r in range(s.nrhs)]
        return {"mfull": mf, "seis": seis, "u": us, "launches": s.launches}


def test_rectangle_matches_oracle():
    m = workloads.build("homogeneous_rectangle", scale=0.25, steps=600)
    o = oracle.run(m, nthreads=NT)
    g = gpu_run(m)
    assert np.array_equal(g["mfull"], o["mfull"])
    assert np.abs(o["seis"]).max() > 1.0
    err = fp64_rel(g["seis"][0], o["seis"])
    assert err.max() <= TOL, err.max()
    assert rel(g["u"][0], o["u"]) <= TOL
    assert g["launches"] > 0


def test_canyon_with_hanging_nodes_every_rhs():
    m = workloads.build("canyon", scale=0.15, steps=700, save_every=2, refine_band=20)
    assert m.problem.nhanging > 0 and m.problem.nrhs == 6
    g = gpu_run(m)
    for r in range(m.problem.nrhs):
        o = oracle.run(m, rhs=r, nthreads=NT)
        assert np.array_equal(g["mfull"], o["mfull"])
        err = fp64_rel(g["seis"][r], o["seis"])
        assert err.max() <= TOL, (r, err.max())
        assert rel(g["u"][r], o["u"]) <= TOL


def test_valley_heterogeneous():
    m = workloads.build("valley", scale=0.12, steps=300, save_every=3)
    o = oracle.run(m, nthreads=NT)
    g = gpu_run(m)
    assert fp64_rel(g["seis"][0], o["seis"]).max() <= TOL


def test_closed_form_variant():
    m = workloads.build("canyon", scale=0.15, steps=400, refine_band=20)
    o = oracle.run(m, rhs=4, nthreads=NT)
    g = gpu_run(m, variant=EXFEM_VARIANT_CLOSED_FORM)
    assert fp64_rel(g["seis"][4], o["seis"]).max() <= 1e-10


def test_graph_chunks_and_numbering_do_not_change_results():
    m = workloads.build("canyon", scale=0.12, steps=130, save_every=1, refine_band=20)
    a = gpu_run(m, use_graph=1, graph_steps=16)
    b = gpu_run(m, use_graph=0)
    c = gpu_run(m, reorder=0)
    with Solver(m) as s:
        s.init_explicit()
        for n in (1, 17, 40, 72):
            s.run(n)
        d = s.seismograms()
    for x in (b["seis"], c["seis"], d):
        assert np.array_equal(a["seis"], x)


def test_full_size_homogeneous_rectangle():
    """256x128 elements, 4000 steps, 64 receivers: every seismogram <= 1e-12."""
    m = workloads.build("homogeneous_rectangle")
    o = oracle.run(m, nthreads=NT)
    g = gpu_run(m)
    err = fp64_rel(g["seis"][0], o["seis"])
    assert err.max() <= TOL, err.max()


def test_call_order_and_argument_errors():
    m = workloads.build("homogeneous_rectangle", scale=0.125, steps=20)
    s = Solver(m)
    with pytest.raises(ExfemError) as e:
        s.run(5)
    assert e.value.code == EXFEM_E_STATE
    s.init_explicit()
    with pytest.raises(ExfemError) as e:
        s.run(21)
    assert e.value.code == EXFEM_E_ARG
    s.run(20)
    s.sync()
    s.close()


def test_post_critical_wave_is_rejected_not_fatal():
    d = decks.homogeneous_rectangle(scale=0.125, steps=10, angle=math.radians(35.0))
    m = Model(d)
    with pytest.raises(ExfemError) as e:
        Solver(m)
    assert e.value.code == EXFEM_E_UNSUPPORTED


@pytest.mark.parametrize("use_graph", [1, 0])
def test_side_stream_drm_forces_match_the_inline_pass_fp64(use_graph):
    """The reference-order FP64 form also computes the next step's DRM
    forces on a second stream by default (exfem_opts.drm_inline = 0): the
    same items in the same order as inside the hanging pass (drm_inline = 1),
    so the results are bit for bit the same, with graph replays mixed with
    single steps and without graphs; and they match the oracle."""
    m = workloads.build("canyon", scale=0.12, steps=130, save_every=1, refine_band=20)
    runs = []
    for inline in (1, 0):
        with Solver(m, drm_inline=inline, use_graph=use_graph) as s:
            s.init_explicit()
            for n in (1, 17, 40, 72):
                s.run(n)
            s.sync()
            runs.append((s.seismograms(), [s.u(r) for r in range(s.nrhs)]))
    assert np.array_equal(runs[0][0], runs[1][0])
    for r in range(m.problem.nrhs):
        assert np.array_equal(runs[0][1][r], runs[1][1][r]), r
    o = oracle.run(m, rhs=3, nthreads=NT)
    assert fp64_rel(runs[1][0][3], o["seis"]).max() <= TOL
