"""Serving (include/exfem_srv.h): continuous batching of uneven requests.

Each request's seismograms must be the same in the mix as alone (FP32 form,
1e-6: the contexts are independent, so in practice they are identical), and
the FP32 results stay within 1e-4 of the FP64 oracle."""
import os

import numpy as np
import pytest

from exfem import decks, workloads
from exfem.abi import EXFEM_E_NOMEM, EXFEM_E_UNSUPPORTED, EXFEM_FP32_KAHAN, EXFEM_FP64
from exfem.gpu import Solver, estimate_bytes
from exfem.model import Model
from exfem.serve import Server, run_stream
from oracle import oracle
from util import per_receiver_rel

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 8


def mix():
    out = []
    for i, (arr, deck, steps) in enumerate(decks.serving_stream(n=6, seed=11, min_scale=0.08, max_scale=0.2,
                                                                 max_angles=4, step_range=(200, 600))):
        out.append((Model(deck, nsteps=steps, io_interval=4), steps))
    return out


def alone32(m, steps):
    with Solver(m, precision=EXFEM_FP32_KAHAN) as s:
        s.init_explicit()
        s.run(steps)
        s.sync()
        return s.seismograms()[:, : steps // m.problem.io_interval + 1]


@pytest.mark.parametrize("tune", [0, 1], ids=["built_in_shapes", "tuned_shapes"])
def test_each_result_is_the_same_in_the_mix_as_alone(tune):
    """With tune = 1 every request's context times its own shapes first
    (exfem_opts.tune): the results are still those of the request alone."""
    reqs = mix()
    with Server(max_active=4, chunk_steps=64, tune=tune) as srv:
        ids = [srv.submit(m, n) for m, n in reqs]
        res = srv.wait_all(len(ids))
        assert len(res) == len(ids) and all(r["status"] == 0 for r in res)
        got = {r["id"]: srv.fetch(r["id"]) for r in res}
        assert srv.stats()["peak_active"] >= 2
    for rid, (m, n) in zip(ids, reqs):
        ref = alone32(m, n)
        for r in range(m.problem.nrhs):
            assert per_receiver_rel(got[rid][r], ref[r]).max() <= 1e-6
    m, n = reqs[0]
    o = oracle.run(m, rhs=0, nsteps=n, nthreads=NT)
    assert per_receiver_rel(got[ids[0]][0], o["seis"]).max() <= 1e-4


def test_admission_respects_the_hbm_budget():
    reqs = mix()
    est = [estimate_bytes(m, precision=EXFEM_FP32_KAHAN) for m, _ in reqs]
    budget = int(sorted(est)[-1] + sorted(est)[-2] + 1)
    with Server(hbm_budget=budget, max_active=8, chunk_steps=64) as srv:
        ids = [srv.submit(m, n) for m, n in reqs]
        res = srv.wait_all(len(ids))
    assert all(r["status"] == 0 for r in res)
    for r in res:   # the reservation bounds what the context really held
        assert r["reserved_bytes"] == est[ids.index(r["id"])] >= r["device_bytes"] > 0
    # at no time do the reservations of running requests exceed the budget
    spans = [(r["t_admit"], r["t_done"], r["reserved_bytes"]) for r in res]
    for t, _, _ in spans:
        assert sum(b for a, d, b in spans if a <= t < d) <= budget


def test_estimate_bounds_every_form_and_copies_are_counted():
    """Admission reserves exfem_gpu_estimate_bytes: it must bound what every
    precision and kernel variant holds, without reserving much more.  The
    context's copy counters see the model upload and the seismogram read."""
    cases = [("canyon", dict(scale=0.2, steps=20)), ("valley_batched", dict(scale=0.1, steps=20)),
             ("point_source", dict(scale=0.5, steps=20, kind="POINTN"))]
    for name, kw in cases:
        m = workloads.build(name, **kw)
        held64 = None
        for prec, variants in ((EXFEM_FP64, (0, 1)), (EXFEM_FP32_KAHAN, (0, 1, 2))):
            for v in variants:
                est = estimate_bytes(m, precision=prec, variant=v)
                s = Solver(m, precision=prec, variant=v)
                s.init_explicit()
                h2d0, d2h0 = s.copy_bytes()
                s.run(4)
                seis = s.seismograms()
                h2d1, d2h1 = s.copy_bytes()
                held = s.device_bytes
                s.close()
                assert est >= held > 0, (name, prec, v, est, held)
                if v == 0 or prec == EXFEM_FP64:
                    # the FP32 tile variants reserve a worst-case halo
                    assert est <= 1.3 * held + (1 << 20), (name, prec, v, est, held)
                assert h2d0 > 0 and h2d1 == h2d0
                assert d2h1 - d2h0 >= seis.nbytes
                if prec == EXFEM_FP64 and v == 0:
                    held64 = held
                if prec == EXFEM_FP32_KAHAN and v == 0 and m.problem.nrhs == 1:
                    # no FP64-only arrays (element operator, own lists, 1/m_full) in an FP32 context
                    assert held < held64


def test_pool_reuse_and_release():
    """Contexts draw their device memory from the library's pool, which keeps
    what destroyed contexts freed: repeated contexts give the same results,
    and after exfem_gpu_release_cached hands the unused memory back, a new
    context allocates afresh and again gives the same results."""
    from exfem.gpu import gpu_lib
    m = workloads.build("canyon", scale=0.2, steps=40)
    outs = []
    for _ in range(3):
        with Solver(m, precision=EXFEM_FP32_KAHAN) as s:
            s.init_explicit()
            s.run()
            s.sync()
            outs.append(s.seismograms())
    assert gpu_lib().exfem_gpu_release_cached(0) == 0
    with Solver(m, precision=EXFEM_FP32_KAHAN) as s:
        s.init_explicit()
        s.run()
        s.sync()
        outs.append(s.seismograms())
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


def test_failures_stay_isolated():
    good, n = mix()[0]
    bad = Model(decks.homogeneous_rectangle(scale=0.125, steps=50, angle=0.6), nsteps=50)   # SV past critical
    with Server(max_active=4) as srv:
        a = srv.submit(good, n)
        b = srv.submit(bad, 50)
        res = {r["id"]: r for r in srv.wait_all(2)}
    assert res[a]["status"] == 0 and res[b]["status"] == EXFEM_E_UNSUPPORTED


def test_request_larger_than_the_budget_is_refused():
    m, n = mix()[1]
    with Server(hbm_budget=4096, max_active=4) as srv:
        rid = srv.submit(m, n)
        res = srv.wait_all(1)
    assert res[0]["id"] == rid and res[0]["status"] == EXFEM_E_NOMEM


def test_timed_stream_reports_latency_and_throughput():
    stream = decks.serving_stream(n=10, rate=40.0, seed=5, min_scale=0.06, max_scale=0.15, max_angles=3,
                                  step_range=(100, 300))
    reqs = [(t, Model(d, nsteps=s, io_interval=4), s) for t, d, s in stream]
    recs, summary, _ = run_stream(reqs, server_kw={"max_active": 6, "chunk_steps": 64})
    assert summary["ok"] == 10 and 0 < summary["p50_s"] <= summary["p99_s"]
    assert summary["throughput"] > 0


def test_deck_requests_match_model_requests():
    """Requests given as problem.in text are meshed by the server's worker
    threads before admission and give the same seismograms as the same
    problems built on the caller's side; a bad deck fails alone."""
    stream = decks.serving_stream(n=4, seed=5, min_scale=0.08, max_scale=0.15, max_angles=3, step_range=(100, 300))
    with Server(max_active=4, chunk_steps=64) as srv:
        ids_deck = [srv.submit_deck(d, n) for _, d, n in stream]
        bad = srv.submit_deck("PROBLEM FILE EXFEM\nDOMAIN:\n-1 -1\n", 10)
        models = [Model(d, nsteps=n) for _, d, n in stream]
        ids_model = [srv.submit(m, n) for m, (_, _, n) in zip(models, stream)]
        res = {r["id"]: r for r in srv.wait_all(2 * len(stream) + 1)}
        assert res[bad]["status"] != 0
        for i in ids_deck:
            r = res[i]
            assert r["status"] == 0
            assert r["t_submit"] <= r["t_meshed"] <= r["t_admit"] <= r["t_ready"] <= r["t_done"]
        got_deck = [srv.fetch(i) for i in ids_deck]
        got_model = [srv.fetch(i) for i in ids_model]
        with pytest.raises(Exception):
            srv.fetch(bad)
    for a, b, (_, _, n) in zip(got_deck, got_model, stream):
        assert a.shape == b.shape and np.array_equal(a, b)


def test_stream_of_decks_reports_latency_with_meshing():
    stream = decks.serving_stream(n=6, rate=40.0, seed=3, min_scale=0.08, max_scale=0.2, max_angles=4,
                                  step_range=(100, 400))
    recs, summary, _ = run_stream(stream, server_kw={"max_active": 4, "chunk_steps": 64})
    assert summary["ok"] == len(stream)
    for r in recs.values():
        assert r["t_meshed"] >= r["t_submit"] and r["latency"] > 0 and r["nelems"] > 0
