"""Point sources (POINTN force, POINTD prescribed displacement) on the GPU
against the CPU oracle, through the C ABI: the FP64 forms at 1e-12 (reference
order) and 1e-10 (closed form), the FP32 form at 1e-4, relative L2 per
receiver seismogram, on the rectangle and on the refined canyon whose source
reaches hanging nodes."""
import os

import numpy as np
import pytest

from exfem import workloads
from exfem.abi import EXFEM_FP32_KAHAN, EXFEM_VARIANT_CLOSED_FORM
from exfem.gpu import Solver
from exfem.serve import Server
from oracle import oracle
from util import fp64_rel, per_receiver_rel, rel

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 8
CASES = [("NONE", "POINTN"), ("CANYON", "POINTN"), ("CANYON", "POINTD"), ("NONE", "POINTD")]


def model(geom, kind, steps=500):
    return workloads.build("point_source", scale=0.15, steps=steps, save_every=2, geom=geom, kind=kind)


def gpu_run(m, **opts):
    with Solver(m, **opts) as s:
        mf = s.init_explicit()
        s.run()
        s.sync()
        return mf, s.seismograms()[0], s.u(0)


@pytest.mark.parametrize("geom,kind", CASES)
def test_fp64_reference_order_matches_oracle(geom, kind):
    m = model(geom, kind)
    o = oracle.run(m, nthreads=NT)
    mf, seis, u = gpu_run(m)
    assert np.array_equal(mf, o["mfull"])
    assert np.abs(o["seis"]).max() > 0
    assert fp64_rel(seis, o["seis"]).max() <= 1e-12
    assert rel(u, o["u"]) <= 1e-12


@pytest.mark.parametrize("geom,kind", CASES[1:3])
def test_fp64_closed_form_matches_oracle(geom, kind):
    m = model(geom, kind)
    o = oracle.run(m, nthreads=NT)
    _, seis, u = gpu_run(m, variant=EXFEM_VARIANT_CLOSED_FORM)
    assert fp64_rel(seis, o["seis"]).max() <= 1e-10
    assert rel(u, o["u"]) <= 1e-10


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("geom,kind", CASES[:3])
def test_fp32_matches_oracle(geom, kind, variant):
    m = model(geom, kind, steps=800)
    o = oracle.run(m, nthreads=NT)
    _, seis, u = gpu_run(m, precision=EXFEM_FP32_KAHAN, variant=variant)
    assert per_receiver_rel(seis, o["seis"]).max() <= 1e-4
    assert rel(u, o["u"]) <= 1e-4


def test_point_requests_are_the_same_served_as_alone():
    reqs = [model("CANYON", "POINTN", 300), model("CANYON", "POINTD", 300), model("NONE", "POINTN", 300)]
    with Server(max_active=3, chunk_steps=32) as srv:
        ids = [srv.submit(m, m.problem.nsteps) for m in reqs]
        res = srv.wait_all(len(ids))
        assert all(r["status"] == 0 for r in res)
        got = {r["id"]: srv.fetch(r["id"]) for r in res}
    for rid, m in zip(ids, reqs):
        _, seis, _ = gpu_run(m, precision=EXFEM_FP32_KAHAN)
        assert per_receiver_rel(got[rid][0], seis).max() <= 1e-6
