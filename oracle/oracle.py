"""ctypes wrapper of the CPU oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU legs; never by
the product.  See exfem_oracle.cpp for what it restates.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "damian.par_gb300"))

from exfem.abi import EXFEM_HANG_HALF, ExfemError, Mesh, Problem  # noqa: E402

from . import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        _build.build_oracle()
        L = C.CDLL(_build.ORACLE_LIB)
        L.oracle_run.restype = C.c_int
        L.oracle_run.argtypes = [C.POINTER(Mesh), C.POINTER(Problem), C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_calck.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.oracle_calcsqm.argtypes = [C.POINTER(C.c_double)]
        L.oracle_multdrm.argtypes = [C.POINTER(C.c_double)] * 2 + [C.POINTER(C.c_ubyte), C.POINTER(C.c_double)]
        L.oracle_planewave.restype = C.c_int
        L.oracle_planewave.argtypes = [C.c_int] + [C.c_double] * 8 + [C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def run(model, rhs=0, nsteps=None, hang_mode=EXFEM_HANG_HALF, nthreads=1, want_u=True):
    """Run the oracle on a built exfem.Model; returns dict(mfull, seis, u, seconds)."""
    p = model.problem
    if nsteps is None:
        nsteps = p.nsteps
    io = max(p.io_interval, 1)
    ndof = 2 * model.nnodes
    mfull = np.zeros(ndof)
    seis = np.zeros((nsteps // io + 1, p.nrecv, 2))
    u = np.zeros(ndof) if want_u else None
    secs = C.c_double(0)
    rc = lib().oracle_run(C.byref(model.mesh), C.byref(p), int(rhs), int(hang_mode), int(nthreads),
                          int(nsteps), _p(mfull), _p(seis), _p(u) if want_u else None, C.byref(secs))
    if rc != 0:
        raise ExfemError(rc, lib().oracle_last_error().decode())
    return {"mfull": mfull, "seis": seis, "u": u, "seconds": secs.value}


def calck(m, l):
    k = np.zeros(64)
    lib().oracle_calck(m, l, _p(k))
    return k.reshape(8, 8, order="F")


def calcsqm():
    k = np.zeros(64)
    lib().oracle_calcsqm(_p(k))
    return k.reshape(8, 8, order="F")


def multdrm(k, u, e):
    kf = np.ascontiguousarray(np.asarray(k, dtype=np.float64).reshape(8, 8).ravel(order="F"))
    uu = np.ascontiguousarray(u, dtype=np.float64)
    ee = np.ascontiguousarray(e, dtype=np.uint8)
    p = np.zeros(8)
    lib().oracle_multdrm(_p(kf), _p(uu), ee.ctypes.data_as(C.POINTER(C.c_ubyte)), _p(p))
    return p


def planewave(kind, amp, alpha, beta, angle, freq, t, x1, x3):
    """Returns (2, 3): rows x/z, columns displacement/velocity/acceleration."""
    out = np.zeros(6)
    rc = lib().oracle_planewave(int(kind), amp, alpha, beta, angle, freq, t, x1, x3, _p(out))
    if rc != 0:
        raise ExfemError(rc, lib().oracle_last_error().decode())
    return out.reshape(3, 2).T
