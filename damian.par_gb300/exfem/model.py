"""Host model: a deck (problem.in text) turned into mesh + problem arrays.

Thin wrapper over ``libexfem_host.so`` (include/exfem_host.h).  The arrays are
exposed as numpy views with the reference's conventions: 1-based indices,
(x, depth) node pairs, interleaved (x, y) dofs.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .abi import (HOST_SYMBOLS, ExfemError, Grid, Mesh, ModelInfo, Problem, bind)

_host = None


def host_lib():
    global _host
    if _host is None:
        _host = bind(_native.load("host"), HOST_SYMBOLS)
    return _host


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).view(dtype)


class Model:
    """A built problem.  Keeps the native model alive while views exist."""

    def __init__(self, deck_text: str, nsteps: int | None = None, io_interval: int | None = None):
        lib = host_lib()
        h = C.c_void_p()
        rc = lib.exfem_model_build(deck_text.encode(), C.byref(h))
        if rc != 0:
            raise ExfemError(rc, lib.exfem_model_error().decode())
        self._h = h
        self.deck = deck_text
        if nsteps is not None and int(nsteps) > 0:
            rc = lib.exfem_model_set_nsteps(h, int(nsteps))
            if rc != 0:
                raise ExfemError(rc, lib.exfem_model_error().decode())
        self.mesh = Mesh()
        self.problem = Problem()
        lib.exfem_model_views(h, C.byref(self.mesh), C.byref(self.problem))
        if io_interval is not None:
            if int(io_interval) < 1:
                raise ExfemError(-1, "io_interval must be >= 1")
            self.problem.io_interval = int(io_interval)   # save_step period (io_utils.f90:390)
        info = ModelInfo()
        lib.exfem_model_get_info(h, C.byref(info))
        self.info = {f: getattr(info, f) for f, _ in ModelInfo._fields_}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                host_lib().exfem_model_free(h)
            except Exception:
                pass
            self._h = None

    # ---- numpy views (read-only by convention) ---------------------------
    @property
    def nelems(self):
        return self.mesh.nelems

    @property
    def nnodes(self):
        return self.mesh.nnodes

    def eptr(self):
        return _arr(self.mesh.eptr, self.mesh.nelems + 1, np.int32)

    def eind(self):
        return _arr(self.mesh.eind, int(self.eptr()[-1]) - 1, np.int32)

    def ediv(self):
        return _arr(self.mesh.ediv, int(self.eptr()[-1]) - 1, np.uint8)

    def nodes(self):
        return _arr(self.mesh.nodes, 2 * self.mesh.nnodes, np.float64).reshape(-1, 2)

    def ematprop(self):
        return _arr(self.mesh.ematprop, self.mesh.nelems, np.int32)

    def matconst(self):
        return _arr(self.problem.matconst, 5 * self.problem.nmat, np.float64).reshape(-1, 5)

    def absorbing(self):
        return _arr(self.problem.absorbing, self.mesh.nnodes, np.int32)

    def hanging(self):
        return _arr(self.problem.hanging, 3 * self.problem.nhanging, np.int32).reshape(-1, 3)

    def seismic(self):
        return _arr(self.problem.seismic, 2 * self.problem.nseismic, np.int32).reshape(-1, 2)

    def receivers(self):
        xy = _arr(self.problem.recv_xy, 2 * self.problem.nrecv, np.float64).reshape(-1, 2)
        el = _arr(self.problem.recv_elem, self.problem.nrecv, np.int32)
        return xy, el

    def waves(self):
        """The right-hand sides' plane waves ([] for a point-source problem)."""
        if not self.problem.waves:
            return []
        return [self.problem.waves[i] for i in range(self.problem.nrhs)]

    def point_nodes(self):
        """1-based point-source nodes (setup_point_source), empty without one."""
        return _arr(self.problem.point_nodes, self.problem.npoint, np.int32)

    def corners(self):
        """Non-hanging corners per element (elemallnhnodes), 1-based, shape (ne, 4)."""
        eptr, eind, ediv = self.eptr(), self.eind(), self.ediv()
        keep = ediv == 0
        cnt = np.add.reduceat(keep.astype(np.int64), eptr[:-1] - 1)
        if not np.all(cnt == 4):
            raise ExfemError(-2, "element without four non-hanging corners")
        return eind[keep].reshape(-1, 4)

    def grid(self, xmin, xmax, ymin, ymax, dist):
        """ANIMAT sampling grid (exfem_model_grid): dict with nx, ny, points
        (n, 2), elem (n,) 1-based or 0, material (n, 2), eptr, eind (1-based
        cells) and nfound."""
        g = C.POINTER(Grid)()
        rc = host_lib().exfem_model_grid(self._h, float(xmin), float(xmax), float(ymin), float(ymax), float(dist),
                                         C.byref(g))
        if rc != 0:
            raise ExfemError(rc, host_lib().exfem_model_error().decode())
        try:
            v = g.contents
            n, nc = v.npoints, v.ncells
            out = {"nx": v.nx, "ny": v.ny, "origin": (v.origin[0], v.origin[1]), "space": v.space,
                   "points": _arr(v.points, 2 * n, np.float64).reshape(-1, 2).copy(),
                   "elem": _arr(v.elem, n, np.int32).copy(),
                   "material": _arr(v.material, 2 * n, np.float64).reshape(-1, 2).copy(),
                   "eptr": _arr(v.eptr, nc + 1, np.int32).copy(),
                   "eind": _arr(v.eind, 4 * nc, np.int32).copy(), "nfound": v.nfound}
        finally:
            host_lib().exfem_grid_free(g)
        return out

    # ---- reference file formats --------------------------------------------
    def save_mesh(self, path):
        rc = host_lib().exfem_model_save_mesh(self._h, str(path).encode())
        if rc != 0:
            raise ExfemError(rc, host_lib().exfem_model_error().decode())

    @property
    def nsave(self):
        p = self.problem
        return p.nsteps // p.io_interval + 1


def write_mass(path, mass):
    m = np.ascontiguousarray(mass, dtype=np.float64)
    rc = host_lib().exfem_write_mass(str(path).encode(), m.size,
                                     m.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise ExfemError(rc, host_lib().exfem_model_error().decode())


def write_step(path, step, u, append=True):
    u = np.ascontiguousarray(u, dtype=np.float64)
    rc = host_lib().exfem_write_step(str(path).encode(), int(bool(append)), int(step), u.size,
                                     u.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise ExfemError(rc, host_lib().exfem_model_error().decode())


def write_sheet(path, points, field, samp):
    """points: (nrecv, 2); field: (nsave, nrecv, 2) — sheet.txt of io.cpp:844-889."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    fld = np.ascontiguousarray(field, dtype=np.float64)
    rc = host_lib().exfem_write_sheet(str(path).encode(), pts.shape[0],
                                      pts.ctypes.data_as(C.POINTER(C.c_double)), fld.shape[0],
                                      fld.ctypes.data_as(C.POINTER(C.c_double)), float(samp))
    if rc != 0:
        raise ExfemError(rc, host_lib().exfem_model_error().decode())


def write_vtu(path, eptr, eind, points, field, name="displacements"):
    """VTK unstructured grid of write_vtk_unst_field (io.cpp:699-842):
    points (n, 2), field (n, 2), 1-based cells eptr/eind."""
    ep = np.ascontiguousarray(eptr, dtype=np.int32)
    ei = np.ascontiguousarray(eind, dtype=np.int32)
    pts = np.ascontiguousarray(points, dtype=np.float64)
    fld = np.ascontiguousarray(field, dtype=np.float64)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rc = host_lib().exfem_write_vtu(str(path).encode(), len(ep) - 1, ip(ep), ip(ei), pts.shape[0], dp(pts),
                                    name.encode(), dp(fld))
    if rc != 0:
        raise ExfemError(rc, host_lib().exfem_model_error().decode())
