"""exfem_gpu_step_noalloc: one FP64 step on device buffers the caller owns.

It is meant for hosts that cannot let the library allocate device memory: a
host whose own pool or arena hands out every device byte up front, or one
with other device work in flight that cudaFree (which synchronizes the whole
device) would stall.  The test keeps its state in torch tensors, steps them
twice in a row through the C ABI and compares each result with the same
steps taken by exfem_gpu_run, within the FP64 parity tolerance of the other
GPU tests (1e-12 relative L2).  It covers three-array rotation on torch's
stream, the aliased two-array form (d_unew = d_um) on the context's stream,
and the restored current device.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import native_probe as npb
from exfem import workloads
from exfem.abi import EXFEM_E_ARG
from exfem.gpu import Solver

pytestmark = pytest.mark.gpu
TOL = 1e-12


def to_internal(plan, model, u_ref_per_rhs):
    """Reference dof order per rhs -> the context's layout ((node*2+d)*R + r)."""
    nn, R = model.nnodes, len(u_ref_per_rhs)
    a = np.stack([u.reshape(nn, 2) for u in u_ref_per_rhs], axis=2)   # (ref node, d, r)
    return np.ascontiguousarray(a[plan.ref_of_node]).ravel()


def to_ref(plan, model, flat):
    nn, R = model.nnodes, model.problem.nrhs
    a = flat.reshape(nn, 2, R)
    out = np.zeros((nn, 2, R))
    out[plan.ref_of_node] = a
    return [out[:, :, r].ravel() for r in range(R)]


CASES = [("homogeneous_rectangle", dict(scale=0.25, steps=400), 330),
         ("canyon", dict(scale=0.12, steps=400, refine_band=20), 300)]


@pytest.mark.parametrize("aliased", [False, True], ids=["three_arrays", "aliased"])
@pytest.mark.parametrize("name,kw,warm", CASES, ids=[c[0] for c in CASES])
def test_step_noalloc_matches_run_twice(name, kw, warm, aliased):
    torch = pytest.importorskip("torch")
    m = workloads.build(name, **kw)
    R = m.problem.nrhs
    plan = npb.PlanView(m)
    ref = Solver(m)
    ref.init_explicit()
    ref.run(warm - 1)
    u_prev = [ref.u(r) for r in range(R)]
    ref.run(1)
    u_cur = [ref.u(r) for r in range(R)]
    assert max(np.abs(u).max() for u in u_cur) > 1e-6       # the wave is in the box

    s = Solver(m)        # only its read-only model arrays are used by the no-alloc step
    s.init_explicit()
    s.sync()
    # three arrays: everything on a torch stream of the test's own, whose
    # handle is passed to the step (so the step is ordered after the uploads
    # and before the read-backs); aliased: the context's own stream (NULL),
    # with device synchronizations around it
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        u = torch.from_numpy(to_internal(plan, m, u_cur)).cuda()
        um = torch.from_numpy(to_internal(plan, m, u_prev)).cuda()
        un = um if aliased else torch.zeros(2 * m.nnodes * R, dtype=torch.float64, device="cuda")
    stream = None if aliased else C.c_void_p(st.cuda_stream)
    if aliased:
        torch.cuda.synchronize()
    for k in (1, 2):
        step = warm + k
        with torch.cuda.stream(st):
            rc = s.lib.exfem_gpu_step_noalloc(s.h, step, C.c_void_p(u.data_ptr()), C.c_void_p(um.data_ptr()),
                                              C.c_void_p(un.data_ptr()), stream)
            assert rc == 0, s.lib.exfem_gpu_last_error(s.h)
            assert torch.cuda.current_device() == 0
            if aliased:
                s.sync()
            got = to_ref(plan, m, un.cpu().numpy())     # on the test's stream: after the step
        ref.run(1)
        for r in range(R):
            want = ref.u(r)
            err = np.linalg.norm(got[r] - want) / np.linalg.norm(want)
            assert err <= TOL, (k, r, err)
        if aliased:
            u, um = un, u                 # e_up = e_u; e_u = new (explicit.f90:147-148), two arrays
            un = um
        else:
            um, u, un = u, un, um         # three-array rotation
    s.close()
    ref.close()


def test_step_noalloc_rejects_models_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    m = workloads.build("canyon", scale=0.6, steps=4)
    drm = 16 * m.problem.nseismic * m.problem.nrhs
    need = 32 + (drm + 3) // 4 * 4 + 8 * m.nelems * m.problem.nrhs
    assert need > 1048576
    s = Solver(m)
    s.init_explicit()
    buf = torch.zeros(2 * m.nnodes * m.problem.nrhs, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    assert s.lib.exfem_gpu_step_noalloc(s.h, 1, p, p, p, None) == EXFEM_E_ARG
    assert b"EXFEM_NOALLOC_SCRATCH_DOUBLES" in s.lib.exfem_gpu_last_error(s.h)
    s.close()
