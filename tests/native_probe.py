"""Test helper: host build of the plan builder and device arithmetic (tests/native/probe.cu)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PKG = os.path.join(REPO, "damian.par_gb300")
sys.path.insert(0, PKG)
from exfem.abi import ExfemError, Mesh, Problem  # noqa: E402

SRC = [os.path.join(HERE, "native", "probe.cu"), os.path.join(PKG, "csrc", "exfem_plan.cpp")]
DEPS = SRC + [os.path.join(PKG, "csrc", f) for f in ("exfem_plan.h", "exfem_device.cuh", "exfem_ctx.h", "exfem_tc.cuh")]
OUT = os.path.join(HERE, "native", "_build", "libprobe.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < max(os.path.getmtime(f) for f in DEPS):
        tmp = OUT + ".tmp%d" % os.getpid()
        cmd = [NVCC, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp",
               "-I", os.path.join(REPO, "include"), "-I", os.path.join(PKG, "csrc"), *SRC, "-o", tmp, "-lgomp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(res.stderr)
        os.replace(tmp, OUT)
    L = C.CDLL(OUT)
    d = C.POINTER(C.c_double)
    L.probe_error.restype = C.c_char_p
    L.probe_q4_ku.argtypes = [C.c_double] * 4 + [d] * 4
    L.probe_q4_ku_corner.argtypes = [C.c_double] * 4 + [d, d, C.c_int, d, d]
    L.probe_q4_corner_acc.argtypes = [C.c_double] * 4 + [d, d, C.c_int, C.c_double, d, d]
    f = C.POINTER(C.c_float)
    L.probe_q4_ku_f32.argtypes = [C.c_float] * 4 + [f] * 4
    L.probe_drm_forces.argtypes = [d, C.c_double, C.c_int, d, d, d]
    L.probe_planewave.restype = C.c_int
    L.probe_planewave.argtypes = [C.c_int] + [C.c_double] * 8 + [d]
    L.probe_planewave32.restype = C.c_int
    L.probe_planewave32.argtypes = [C.c_int] + [C.c_double] * 8 + [f, f]
    L.probe_planewave_u.restype = C.c_int
    L.probe_planewave_u.argtypes = [C.c_int] + [C.c_double] * 8 + [d]
    L.probe_plan.restype = C.c_void_p
    L.probe_plan.argtypes = [C.POINTER(Mesh), C.POINTER(Problem), C.c_int]
    L.probe_plan_free.argtypes = [C.c_void_p]
    L.probe_set_threads.argtypes = [C.c_int]
    L.probe_state_at.restype = C.c_longlong
    L.probe_state_at.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_int, C.c_int]
    L.probe_calck_check.restype = C.c_int
    L.probe_calck_check.argtypes = [C.c_double, C.c_double]
    L.probe_plan_size.restype = C.c_longlong
    L.probe_plan_size.argtypes = [C.c_void_p, C.c_char_p]
    L.probe_plan_copy.restype = C.c_int
    L.probe_plan_copy.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
    L.probe_tiles.restype = C.c_int
    L.probe_tiles.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)] + [C.c_void_p] * 5
    L.probe_tile_runs.restype = C.c_int
    L.probe_pipe_pack.restype = C.c_int
    L.probe_pipe_pack.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)] + [C.c_void_p] * 4
    L.probe_tile_runs.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.probe_mma_tiles.restype = C.c_int
    L.probe_mma_tiles.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)] + [C.c_void_p] * 4
    L.probe_node_slots.restype = C.c_longlong
    L.probe_node_slots.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.probe_node_coef32.restype = None
    L.probe_node_coef32.argtypes = [C.c_void_p, C.c_void_p]
    L.probe_mma_btile.restype = None
    L.probe_mma_btile.argtypes = [C.c_void_p]
    L.probe_plan_wave.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, d]
    _lib = L
    return L


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


INT_FIELDS = {"ref_of_node", "node_of_ref", "ref_of_elem", "econn", "edamp", "tptr", "tlist", "dptr", "dlist",
              "hang", "s_elem", "s_kind", "rnode", "rsoil", "lptr", "llist", "ownptr", "ownlist", "elem_of_ref",
              "odptr", "odlist"}
FLOAT32_FIELDS = {"ecoef32", "ecoef2"}


class PlanView:
    """All arrays of a host-built plan, as numpy arrays."""

    def __init__(self, model, reorder=True):
        L = lib()
        self.h = L.probe_plan(C.byref(model.mesh), C.byref(model.problem), int(reorder))
        if not self.h:
            raise ExfemError(-1, L.probe_error().decode())
        self.model = model

    def __getattr__(self, name):
        if name.startswith("_") or name in ("h", "model"):
            raise AttributeError(name)
        L = lib()
        n = L.probe_plan_size(self.h, name.encode())
        if n < 0:
            raise AttributeError(name)
        dtype = np.int32 if name in INT_FIELDS else (np.float32 if name in FLOAT32_FIELDS else np.float64)
        out = np.zeros(max(n, 1), dtype=dtype)
        L.probe_plan_copy(self.h, name.encode(), out.ctypes.data_as(C.c_void_p))
        out = out[:n]
        self.__dict__[name] = out
        return out

    def tiles(self, tn):
        """(hptr, hlist, tslot (nterms, 4), nslot, lslot, hmax) of build_tiles."""
        L = lib()
        sz = (C.c_int * 4)()
        assert L.probe_tiles(self.h, tn, sz, None, None, None, None, None) == 0
        nt, hmax, nh = sz[0], sz[1], sz[2]
        hptr = np.zeros(nt + 1, np.int32)
        hlist = np.zeros(max(nh, 1), np.int32)
        tslot = np.zeros(4 * len(self.tlist), np.uint16)
        nslot = np.zeros(int(self.scalars[0]), np.int32)
        lslot = np.zeros(max(len(self.llist) // 2, 1), np.int32)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        assert L.probe_tiles(self.h, tn, sz, vp(hptr), vp(hlist), vp(tslot), vp(nslot), vp(lslot)) == 0
        return hptr, hlist[:nh], tslot.reshape(-1, 4), nslot, lslot[:len(self.llist) // 2], hmax

    def mma_tiles(self, tn=32, emax=64):
        """(nptr, eptr, elist, tj) of build_mma_tiles, or None when refused."""
        L = lib()
        sz = (C.c_int * 3)()
        if L.probe_mma_tiles(self.h, tn, emax, sz, None, None, None, None) != 0:
            return None
        nt, nel = sz[0], sz[1]
        nptr = np.zeros(nt + 1, np.int32)
        eptr = np.zeros(nt + 1, np.int32)
        elist = np.zeros(max(nel, 1), np.int32)
        tj = np.zeros(max(len(self.tlist), 1), np.uint8)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        assert L.probe_mma_tiles(self.h, tn, emax, sz, vp(nptr), vp(eptr), vp(elist), vp(tj)) == 0
        return nptr, eptr, elist[:nel], tj[:len(self.tlist)]

    def node_slots(self):
        """(slot4 (n_active, 4), invm, marked) of build_node_slots, and the
        node coefficients (n_active, 4) of node_coef32."""
        L = lib()
        na = int(self.scalars[0])
        slot4 = np.zeros((max(na, 1), 4), np.int32)
        invm = np.zeros(max(na, 1), np.float32)
        nc = np.zeros((max(na, 1), 4), np.float32)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        marked = L.probe_node_slots(self.h, vp(slot4), vp(invm))
        assert marked >= 0
        L.probe_node_coef32(self.h, vp(nc))
        return slot4[:na], invm[:na], int(marked), nc[:na]

    def tile_runs(self, tn):
        """(rptr, runs (nruns, 2) as (first node, count)) of build_tiles."""
        L = lib()
        nr = L.probe_tile_runs(self.h, tn, None, None)
        assert nr >= 0
        nt = (int(self.scalars[0]) + tn - 1) // tn
        rptr = np.zeros(nt + 1, np.int32)
        runs = np.zeros(max(2 * nr, 2), np.int32)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        assert L.probe_tile_runs(self.h, tn, vp(rptr), vp(runs)) == nr
        return rptr, runs[:2 * nr].reshape(-1, 2)

    def pipe_pack(self, tn, max_runs=64):
        """(hdr (ntiles, 4), runs (ntiles, max_runs, 2), nrec (n_active, 8),
        tpack, tmax) of build_pipe_pack, or None when the model does not fit."""
        L = lib()
        sz = (C.c_int * 5)()
        rc = L.probe_pipe_pack(self.h, tn, max_runs, sz, None, None, None, None)
        if rc == 1:
            return None
        assert rc == 0
        arrs = [np.zeros(max(sz[i], 1), np.int32) for i in range(4)]
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        assert L.probe_pipe_pack(self.h, tn, max_runs, sz, *[vp(a) for a in arrs]) == 0
        hdr, runs, nrec, tpack = [a[:sz[i]] for i, a in enumerate(arrs)]
        return hdr.reshape(-1, 4), runs.reshape(-1, max_runs, 2), nrec.reshape(-1, 8), tpack, sz[4]

    def wave(self, r, t, x1, x3):
        out = np.zeros(6)
        lib().probe_plan_wave(self.h, r, t, x1, x3, dp(out))
        return out

    def __del__(self):
        h = self.__dict__.get("h")
        if h:
            lib().probe_plan_free(h)
