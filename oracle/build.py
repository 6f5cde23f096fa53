"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libexfem_oracle.so`` — the C++ restatement in
  exfem_oracle.cpp (FP64, -ffp-contract=off so x86 and Arm round alike).
* ``oracle/_ref/libref_io.so`` — the reference's own ``io.cpp`` (problem.in
  parser and mesh/mass/step/sheet file I/O), compiled unchanged from the
  read-only reference tree (``EXFEM_REFERENCE_TREE``) when that tree is
  present.  It pins the file
  formats and the deck parser; the solver itself cannot be compiled (Fortran,
  MPI, ParMETIS and ACML are absent, and model.f90:643 does not compile).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(BUILD, "libexfem_oracle.so")
REF_IO_LIB = os.path.join(REF_OUT, "libref_io.so")
# where the reference's source tree is mounted read-only (absent on GPU hosts)
REFERENCE_TREE = os.environ.get("EXFEM_REFERENCE_TREE", "/root/reference")


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "exfem_oracle.cpp")
    hdr = os.path.join(REPO, "include", "exfem_gpu.h")
    if (not force and os.path.exists(ORACLE_LIB)
            and os.path.getmtime(ORACLE_LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return ORACLE_LIB
    tmp = ORACLE_LIB + ".tmp%d" % os.getpid()
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-I", os.path.join(REPO, "include"), src, "-o", tmp])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_ref_io(force=False):
    """Compile the reference's io.cpp where the reference tree exists (not on
    GPU hosts).  Returns the library path or None."""
    src = os.path.join(REFERENCE_TREE, "io.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    if not force and os.path.exists(REF_IO_LIB) and os.path.getmtime(REF_IO_LIB) >= os.path.getmtime(src):
        return REF_IO_LIB
    tmp = REF_IO_LIB + ".tmp%d" % os.getpid()
    _run(["g++", "-O2", "-fPIC", "-shared", "-w", "-I", REFERENCE_TREE, src, "-o", tmp])
    os.replace(tmp, REF_IO_LIB)
    return REF_IO_LIB


def build_all(force=False):
    build_oracle(force)
    build_ref_io(force)


if __name__ == "__main__":
    build_all(force=True)
    print(ORACLE_LIB)
