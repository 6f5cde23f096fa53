"""Build and load the native libraries of the exfem GB300 path.

Two shared objects make up the product:

* ``libexfem_host.so`` — the host side (deck parsing, quadtree mesher, model
  setup), the role the Fortran host plays in damian.par (main.f90:42-53).
* ``libexfem_gpu.so`` — the CUDA time-stepping library behind the C ABI of
  ``include/exfem_gpu.h`` (replaces explicit.f90:79-159).

Both are compiled in-tree into ``damian.par_gb300/_build`` for sm_103a.  There
is no fallback: loading fails loudly when a library is missing.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # damian.par_gb300/
REPO = os.path.dirname(PKG_DIR)
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG_DIR, "_build")
CSRC = os.path.join(PKG_DIR, "csrc")
HOST_SRC = os.path.join(PKG_DIR, "host")

HOST_LIB = os.path.join(BUILD, "libexfem_host.so")
GPU_LIB = os.path.join(BUILD, "libexfem_gpu.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

_lock = threading.Lock()
_libs: dict[str, ctypes.CDLL] = {}


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def host_sources():
    return [os.path.join(HOST_SRC, "exfem_model.cpp"), os.path.join(INCLUDE, "exfem_host.h"),
            os.path.join(INCLUDE, "exfem_gpu.h")]


def gpu_sources():
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp", ".cuh", ".h")))
    return srcs + sorted(os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")) + [HOST_LIB]


def build_host(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and _newer(HOST_LIB, host_sources()):
        return HOST_LIB
    tmp = HOST_LIB + ".tmp%d" % os.getpid()
    # no a*b+c contraction (g++ contracts on aarch64 by default): the mesher's
    # geometric tests give the same mesh on every machine
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-fopenmp", "-ffp-contract=off", "-I", INCLUDE,
          os.path.join(HOST_SRC, "exfem_model.cpp"), "-o", tmp])
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


def build_gpu(force=False):
    """Compile every .cu/.cpp of csrc/ for sm_103a in parallel and link the .so
    (against the host library, which it needs for the server's decks)."""
    build_host(force)
    os.makedirs(BUILD, exist_ok=True)
    if not force and _newer(GPU_LIB, gpu_sources()):
        return GPU_LIB
    units = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    objs = []

    def compile_unit(f):
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        # host code never contracts a*b+c (g++ does on aarch64 by default),
        # so host-side FP64 setup rounds like the CPU oracle on both machines
        host = ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp"]
        if f.endswith(".cu"):
            # *_nofma.cu keep the reference's separate roundings on the device
            fmad = ["-fmad=false"] if f.endswith("_nofma.cu") else []
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", *fmad, *host,
                   "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        else:
            cmd = [NVCC, "-O3", "-std=c++17", *host, "-I", INCLUDE, "-I", CSRC,
                   "-c", src, "-o", obj]
        _run(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, max(1, len(units)))) as ex:
        objs = list(ex.map(compile_unit, units))
    tmp = GPU_LIB + ".tmp%d" % os.getpid()
    # the server meshes decks with the host library, found beside this one
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-L", BUILD, "-lexfem_host", "-Xlinker", "-rpath",
          "-Xlinker", "$ORIGIN", "-lcudart", "-lgomp"])
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


def build_all(force=False):
    build_host(force)
    build_gpu(force)


def load(name):
    """Load one of 'host' / 'gpu'.  Raises when the library has not been built."""
    path = {"host": HOST_LIB, "gpu": GPU_LIB}[name]
    with _lock:
        lib = _libs.get(name)
        if lib is None:
            if not os.path.exists(path):
                raise OSError("exfem native library missing: %s (run __graft_entry__.build())" % path)
            lib = ctypes.CDLL(path)
            _libs[name] = lib
        return lib
