"""Autotuner for the FP32 step kernel.

Tries (kernel variant, block size, right-hand sides per thread) on the real
model — variant 0 is the direct gather, 1 the shared-memory tiled kernel,
2 the persistent kernel fed by bulk copies (needs nrhs a multiple of 4).
Each candidate gets its own context, a few warm-up steps and a
CUDA-event-timed burst on the library's stream; the fastest wins.  Results
are cached per (elements, nodes, rhs) in-process.
"""
from __future__ import annotations

import ctypes as C

from .abi import EXFEM_FP32_KAHAN, ExfemError
from .gpu import Solver

_cache: dict = {}


def candidates(R):
    rpts = [r for r in (1, 2, 4) if R % r == 0]
    vs = (0, 1, 2) if R % 4 == 0 else (0, 1)
    return [(v, bt, r) for v in vs for r in rpts for bt in (128, 256, 512)]


def tune(model, steps=12, warmup=3, device=0, verbose=False):
    key = (model.nelems, model.nnodes, model.problem.nrhs)
    if key in _cache:
        return _cache[key]
    R = model.problem.nrhs
    best = None
    results = []
    need = warmup + steps
    if model.problem.nsteps < need:
        raise ExfemError(-1, "autotune needs %d steps in the model" % need)
    for var, bt, rpt in candidates(R):
        try:
            s = Solver(model, precision=EXFEM_FP32_KAHAN, device=device, block_threads=bt, rhs_per_thread=rpt,
                       use_graph=0, variant=var)
        except ExfemError:
            continue
        try:
            s.init_explicit()
            s.run(warmup)
            s.sync()
            ms = C.c_double(0)
            rc = s.lib.exfem_gpu_run_timed(s.h, steps, C.byref(ms))
        except ExfemError:
            rc = -1
        finally:
            s.close()
        if rc != 0:
            continue
        results.append((ms.value / steps, var, bt, rpt))
        if best is None or ms.value < best[0]:
            best = (ms.value, var, bt, rpt)
    if verbose:
        for r in sorted(results):
            print("autotune: %.4f ms/step variant %d block %d rhs/thread %d" % r)
    choice = {"variant": best[1], "block_threads": best[2], "rhs_per_thread": best[3],
              "ms_per_step": best[0] / steps,
              "tried": [{"ms_per_step": a, "variant": v, "block_threads": b, "rhs_per_thread": c}
                        for a, v, b, c in sorted(results)]}
    _cache[key] = choice
    return choice
