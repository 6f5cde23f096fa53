"""The plan builder's parallel passes give the arrays of a serial build.

build_plan (damian.par_gb300/csrc/exfem_plan.cpp) fills its arrays with
OpenMP loops: the Morton radix sorts, the incidence lists (atomic placement,
then each node's entries ordered by reference element), CSR pointers by
chunked prefix sums, the dashpot slot numbering and the first-error
reductions.  Every array must be the same whatever the thread count, and the
same as the single-threaded builder it replaced: the digests below were taken
from that builder on the same decks, over every array but the FP32 element
coefficients, whose definition changed after it (two stored values, the four
derived from them: test_fp32_coefficients_derive_from_two_values).
"""
import hashlib
import os

import numpy as np
import pytest

import native_probe as npb
from exfem import workloads

FIELDS = ["ref_of_node", "node_of_ref", "ref_of_elem", "elem_of_ref", "econn", "ecoef", "emulam",
          "emass", "edamp", "edampv", "tptr", "tlist", "dptr", "dlist", "mfull_ref", "inv_mfull", "mfull_int",
          "nmass", "ndamp", "hang", "s_elem", "s_kind", "rnode", "rw", "rsoil", "rxy", "lptr", "llist",
          "ownptr", "ownlist", "odptr", "odlist", "nxy", "scalars"]

# (workload, kwargs) -> digest of the single-threaded builder's arrays
CASES = {
    "valley_batched": (dict(scale=0.12, steps=20), "e8ae93a9acd63b93"),
    "canyon": (dict(scale=0.2, steps=10), "6a605c372974b03d"),
    "point_source": (dict(scale=0.5, steps=10, kind="POINTD"), "5c5796d8eeab0f67"),
    "homogeneous_rectangle": (dict(scale=0.5, steps=10), "7233fd701507a698"),
    # large enough for several sort and prefix-sum chunks per pass
    "valley": (dict(scale=0.45, steps=10), "b75f38965511ea6c"),
    "canyon@large": (dict(scale=0.9, steps=10), "5d5f7462b2b92b59"),
}


def plan_digest(P):
    h = hashlib.sha256()
    for f in FIELDS:
        a = np.ascontiguousarray(getattr(P, f))
        h.update(f.encode())
        h.update(str(a.dtype).encode())
        h.update(a.tobytes())
    return h.hexdigest()[:16]


@pytest.mark.parametrize("name", sorted(CASES))
def test_plan_same_for_every_thread_count(name):
    kw, pinned = CASES[name]
    m = workloads.build(name.split("@")[0], **kw)
    L = npb.lib()
    digests = {}
    try:
        for t in (1, 3, 8):
            L.probe_set_threads(t)
            P = npb.PlanView(m)
            digests[t] = plan_digest(P)
            del P
    finally:
        L.probe_set_threads(os.cpu_count() or 1)
    assert len(set(digests.values())) == 1, digests
    assert digests[1] == pinned, digests


def test_plan_errors_name_the_first_bad_element():
    """The parallel validation reports the lowest failing element, as the
    serial scan did."""
    m = workloads.build("homogeneous_rectangle", scale=0.25, steps=5)
    ematprop = m.ematprop()   # a view of the model's own array
    saved = ematprop.copy()
    L = npb.lib()
    try:
        ematprop[[700, 41, 300]] = 99   # out of range: elements 42, 301, 701 (1-based)
        for t in (1, 8):
            L.probe_set_threads(t)
            assert not L.probe_plan(m.mesh, m.problem, 1)
            assert L.probe_error().decode() == "ematprop out of range in element 42"
    finally:
        ematprop[:] = saved
        L.probe_set_threads(os.cpu_count() or 1)
    h = L.probe_plan(m.mesh, m.problem, 1)
    assert h
    L.probe_plan_free(h)


def test_fp32_coefficients_derive_from_two_values():
    """The FP32 form stores two values per element, lambda/12 and mu/4, each
    rounded once from FP64, and derives its four closed-form coefficients from
    them with single FP32 operations (fp32_coef, exfem_plan.h; the device's
    coef_from2 does the same): B = 3 b3, A = B + 2 c, D = b3 + c.  Each is
    within 2 ulps of its FP64 value ((l+2m)/4, l/4, m/4, (l+3m)/12)."""
    f = np.float32
    for name in ("valley", "canyon"):
        m = workloads.build(name, scale=0.3, steps=4)
        P = npb.PlanView(m)
        e2 = np.asarray(P.ecoef2).reshape(-1, 2)
        e4 = np.asarray(P.ecoef32).reshape(-1, 4)
        mulam = np.asarray(P.emulam).reshape(-1, 2)
        mu, lam = mulam[:, 0], mulam[:, 1]
        assert np.array_equal(e2[:, 0], (lam / 12.0).astype(f)) and np.array_equal(e2[:, 1], (mu / 4.0).astype(f))
        B = f(3) * e2[:, 0]
        want = np.stack([B + f(2) * e2[:, 1], B, e2[:, 1], e2[:, 0] + e2[:, 1]], axis=1)
        assert np.array_equal(e4, want)
        exact = np.stack([(lam + 2 * mu) / 4, lam / 4, mu / 4, (lam + 3 * mu) / 12], axis=1)
        ulp = np.spacing(exact.astype(f)).astype(np.float64)
        assert np.all(np.abs(e4.astype(np.float64) - exact) <= 2 * ulp)
        assert np.array_equal(np.asarray(P.ecoef).reshape(-1, 4), exact)
