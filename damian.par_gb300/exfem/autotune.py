"""Autotuner for the FP32 step kernel: a binding of exfem_gpu_autotune.

The library times every candidate (kernel variant, block size, right-hand
sides per thread) on the real model — variant 0 is the direct gather, 4 the
same as a persistent grid, 5 its list form (from 50,000 nodes, where 0 reads
fixed-size node records), 1 the shared-memory tiled kernel, 2 the persistent
kernel fed by bulk copies (when nrhs is a multiple of 4), 3 the tensor-core
step (when nrhs is a multiple of 16) — each in a context of its own, with
CUDA events on its stream, and keeps the fastest.  Results are cached in the process per
(elements, nodes, rhs, device), inside the library, so a Fortran host or the
server gets the same shapes as this module.
"""
from __future__ import annotations

import ctypes as C

from .abi import EXFEM_FP32_KAHAN, ExfemError
from .gpu import default_opts, gpu_lib


def tune(model, steps=12, warmup=3, device=0, verbose=False):
    """{variant, block_threads, rhs_per_thread, ms_per_step} for this model.
    `warmup` is the library's (3 steps); kept for the callers' signature."""
    lib = gpu_lib()
    o = default_opts(precision=EXFEM_FP32_KAHAN, device=device)
    ms = C.c_double(0)
    rc = lib.exfem_gpu_autotune(C.byref(model.mesh), C.byref(model.problem), C.byref(o), int(steps), C.byref(ms))
    if rc != 0:
        raise ExfemError(rc, "exfem_gpu_autotune failed")
    choice = {"variant": o.variant, "block_threads": o.block_threads, "rhs_per_thread": o.rhs_per_thread,
              "ms_per_step": ms.value}
    if verbose:
        print("autotune: %.4f ms/step variant %d block %d rhs/thread %d"
              % (ms.value, o.variant, o.block_threads, o.rhs_per_thread))
    return choice
