"""The plan builder's parallel passes give the arrays of a serial build.

build_plan (damian.par_gb300/csrc/exfem_plan.cpp) fills its arrays with
OpenMP loops: the Morton radix sorts, the incidence lists (atomic placement,
then each node's entries ordered by reference element), CSR pointers by
chunked prefix sums, the dashpot slot numbering and the first-error
reductions.  Every array must be the same whatever the thread count, and the
same as the single-threaded builder it replaced: the digests below were taken
from that builder on the same decks.
"""
import hashlib
import os

import numpy as np
import pytest

import native_probe as npb
from exfem import workloads

FIELDS = ["ref_of_node", "node_of_ref", "ref_of_elem", "elem_of_ref", "econn", "ecoef", "ecoef32", "emulam",
          "emass", "edamp", "edampv", "tptr", "tlist", "dptr", "dlist", "mfull_ref", "inv_mfull", "mfull_int",
          "nmass", "ndamp", "hang", "s_elem", "s_kind", "rnode", "rw", "rsoil", "rxy", "lptr", "llist",
          "ownptr", "ownlist", "odptr", "odlist", "nxy", "scalars"]

# (workload, kwargs) -> digest of the single-threaded builder's arrays
CASES = {
    "valley_batched": (dict(scale=0.12, steps=20), "26a6c1bfb9cabadc"),
    "canyon": (dict(scale=0.2, steps=10), "fa53144bef79ac0b"),
    "point_source": (dict(scale=0.5, steps=10, kind="POINTD"), "4e235952da0c6b34"),
    "homogeneous_rectangle": (dict(scale=0.5, steps=10), "4b81df71342c039c"),
    # large enough for several sort and prefix-sum chunks per pass
    "valley": (dict(scale=0.45, steps=10), "bf51c2b72f8a59f6"),
    "canyon@large": (dict(scale=0.9, steps=10), "b96363ed79b27238"),
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
