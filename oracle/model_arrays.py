"""A built model as plain arrays, for the oracle's timed CPU runs (test
infrastructure only).

`dump` writes a model's mesh and problem arrays (the contents of the
exfem_mesh / exfem_problem structs of include/exfem_gpu.h) to an .npz file;
`load` rebuilds those structs over numpy arrays, which is all `oracle.run`
reads.  bench.py's reference arm meshes its workload in a child process that
calls `dump`, then loads the file, so the process it times maps the oracle
and nothing of the product's native libraries.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "damian.par_gb300"))

from exfem.abi import Mesh, Problem, Wave  # noqa: E402  (ctypes declarations only)

_SCALARS = ("nmat", "nhanging", "nseismic", "deltat", "nsteps", "io_interval", "walpha", "wbeta", "nrhs",
            "nrecv", "point_kind", "npoint", "point_amp", "point_sigma", "point_t0")


def dump(model, path):
    p = model.problem
    waves = model.waves()
    arrays = {
        "eptr": model.eptr(), "eind": model.eind(), "ediv": model.ediv(), "nodes": model.nodes().ravel(),
        "ematprop": model.ematprop(), "matconst": model.matconst().ravel(), "absorbing": model.absorbing(),
        "hanging": model.hanging().ravel(), "seismic": model.seismic().ravel(),
        "recv_xy": model.receivers()[0].ravel(), "recv_elem": model.receivers()[1],
        "point_nodes": model.point_nodes(),
        "waves": np.array([[w.kind, w.amp, w.angle, w.freq, w.t0] for w in waves], dtype=np.float64).reshape(-1, 5),
        "worigin": np.array(list(p.worigin)), "wbox": np.array(list(p.wbox)),
        "scalars": np.array([float(getattr(p, k)) for k in _SCALARS]),
        "sizes": np.array([model.nelems, model.nnodes]),
    }
    np.savez(path, **arrays)


class ArrayModel:
    """The exfem_mesh / exfem_problem structs over arrays loaded from `dump`."""

    def __init__(self, path):
        d = np.load(path)
        self._keep = {}

        def arr(name, dtype):
            a = np.ascontiguousarray(d[name], dtype=dtype)
            self._keep[name] = a
            return a

        ne, nn = (int(v) for v in d["sizes"])
        self.mesh = Mesh()
        self.mesh.nelems, self.mesh.nnodes = ne, nn
        self.mesh.eptr = arr("eptr", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        self.mesh.eind = arr("eind", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        self.mesh.ediv = arr("ediv", np.uint8).ctypes.data_as(C.POINTER(C.c_ubyte))
        self.mesh.nodes = arr("nodes", np.float64).ctypes.data_as(C.POINTER(C.c_double))
        self.mesh.ematprop = arr("ematprop", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        p = Problem()
        for k, v in zip(_SCALARS, d["scalars"]):
            setattr(p, k, int(v) if isinstance(getattr(p, k), int) else float(v))
        p.matconst = arr("matconst", np.float64).ctypes.data_as(C.POINTER(C.c_double))
        p.absorbing = arr("absorbing", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        p.hanging = arr("hanging", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        p.seismic = arr("seismic", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        p.recv_xy = arr("recv_xy", np.float64).ctypes.data_as(C.POINTER(C.c_double))
        p.recv_elem = arr("recv_elem", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        p.point_nodes = arr("point_nodes", np.int32).ctypes.data_as(C.POINTER(C.c_int))
        for i, v in enumerate(d["worigin"]):
            p.worigin[i] = float(v)
        for i, v in enumerate(d["wbox"]):
            p.wbox[i] = float(v)
        wv = d["waves"]
        if len(wv):
            warr = (Wave * len(wv))()
            for i, (kind, amp, angle, freq, t0) in enumerate(wv):
                warr[i] = Wave(int(kind), amp, angle, freq, t0)
            self._keep["waves"] = warr
            p.waves = C.cast(warr, C.POINTER(Wave))
        self.problem = p

    @property
    def nelems(self):
        return self.mesh.nelems

    @property
    def nnodes(self):
        return self.mesh.nnodes
