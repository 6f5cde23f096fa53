"""Python view of the C ABI in include/exfem_gpu.h (the drop-in for
init_explicit/run_explicit, explicit.f90:79-159).

    from exfem import decks
    from exfem.model import Model
    from exfem.gpu import Solver
    m = Model(decks.homogeneous_rectangle())
    with Solver(m) as s:
        mfull = s.init_explicit()
        s.run()                      # all of the problem's steps
        seis = s.seismograms()       # (nrhs, nsave, nrecv, 2)

Every call goes through libexfem_gpu.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .abi import (EXFEM_FP32_KAHAN, EXFEM_FP64, GPU_SYMBOLS, ExfemError, Opts, bind)

_gpu = None


def gpu_lib():
    global _gpu
    if _gpu is None:
        _gpu = bind(_native.load("gpu"), GPU_SYMBOLS)
    return _gpu


def default_opts(**kw):
    o = Opts()
    gpu_lib().exfem_gpu_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError("unknown option %r" % k)
        setattr(o, k, int(v))
    return o


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Solver:
    """One device-resident problem (exfem_ctx)."""

    def __init__(self, model, precision=EXFEM_FP64, **opts):
        self.model = model
        self.lib = gpu_lib()
        self.opts = default_opts(precision=precision, **opts)
        h = C.c_void_p()
        rc = self.lib.exfem_gpu_create(C.byref(model.mesh), C.byref(model.problem), C.byref(self.opts), C.byref(h))
        if rc != 0:
            raise ExfemError(rc, self.lib.exfem_gpu_last_error(None).decode())
        self.h = h
        self.nrhs = model.problem.nrhs
        self.nrecv = model.problem.nrecv
        self.io = model.problem.io_interval
        self.nsteps = model.problem.nsteps

    def _check(self, rc):
        if rc != 0:
            raise ExfemError(rc, self.lib.exfem_gpu_last_error(self.h).decode())

    def init_explicit(self, want_mfull=True):
        """init_explicit; returns m_full (mass.bin's content), or None with
        want_mfull False (no host copy of it)."""
        if not want_mfull:
            self._check(self.lib.exfem_gpu_init_explicit(self.h, None))
            return None
        mfull = np.zeros(2 * self.model.nnodes)
        self._check(self.lib.exfem_gpu_init_explicit(self.h, _dp(mfull)))
        return mfull

    def run(self, nsteps=None):
        if nsteps is None:
            nsteps = self.nsteps - self.steps_done
        self._check(self.lib.exfem_gpu_run(self.h, int(nsteps)))

    def sync(self):
        self._check(self.lib.exfem_gpu_sync(self.h))

    @property
    def steps_done(self):
        return self.lib.exfem_gpu_steps_done(self.h)

    @property
    def launches(self):
        return self.lib.exfem_gpu_launch_count(self.h)

    @property
    def device_bytes(self):
        return self.lib.exfem_gpu_device_bytes(self.h)

    def copy_bytes(self):
        """(host -> device, device -> host) bytes the context has copied so far."""
        h2d, d2h = C.c_ulonglong(), C.c_ulonglong()
        self._check(self.lib.exfem_gpu_copy_bytes(self.h, C.byref(h2d), C.byref(d2h)))
        return int(h2d.value), int(d2h.value)

    def kernel_times(self, steps):
        """{kernel name: mean ms per launch} over `steps` steps run without a
        graph (CUDA events between launches on the context's stream)."""
        ms = (C.c_double * 16)()
        nm = (C.c_char_p * 16)()
        nk = self.lib.exfem_gpu_profile_kernels(self.h, int(steps), ms, nm, 16)
        if nk < 0:
            self._check(nk)
        return {nm[i].decode(): ms[i] for i in range(nk)}

    def sample_points(self, xy, elem, rhs=0):
        """visu_field at points (n, 2) in 1-based elements (0: none) for the
        current step: (n, 2) displacements."""
        pts = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        el = np.ascontiguousarray(elem, dtype=np.int32)
        out = np.zeros((pts.shape[0], 2))
        self._check(self.lib.exfem_gpu_sample_points(self.h, int(rhs), pts.shape[0], _dp(pts),
                                                     el.ctypes.data_as(C.POINTER(C.c_int)), _dp(out)))
        return out

    def u(self, rhs=0):
        out = np.zeros(2 * self.model.nnodes)
        self._check(self.lib.exfem_gpu_get_u(self.h, int(rhs), _dp(out), out.size))
        return out

    def seismograms(self, out=None):
        """(nrhs, nsave_total, nrecv, 2); rows past the steps done are zero."""
        nsave = self.nsteps // self.io + 1
        if out is None:
            out = np.zeros((self.nrhs, nsave, self.nrecv, 2))
        ns = C.c_int(0)
        self._check(self.lib.exfem_gpu_get_seismograms(self.h, _dp(out), out.size, C.byref(ns)))
        return out

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.exfem_gpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_bytes(model, precision=EXFEM_FP64, **opts):
    o = default_opts(precision=precision, **opts)
    return gpu_lib().exfem_gpu_estimate_bytes(C.byref(model.mesh), C.byref(model.problem), C.byref(o))


__all__ = ["Solver", "default_opts", "estimate_bytes", "EXFEM_FP64", "EXFEM_FP32_KAHAN"]
