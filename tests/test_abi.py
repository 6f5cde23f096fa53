"""The C-ABI libraries load and export every symbol their headers declare
(no compute call: these run without a GPU)."""
import ctypes as C
import os
import re

from exfem import _native
from exfem.abi import EXFEM_E_ARG, Mesh, Opts, Problem

INC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared(header):
    txt = open(os.path.join(INC, header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(exfem_\w+)\s*\(", txt)))


def test_gpu_library_exports_header_symbols():
    lib = C.CDLL(_native.GPU_LIB)
    names = declared("exfem_gpu.h")
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n


def test_server_symbols_are_exported():
    lib = C.CDLL(_native.GPU_LIB)
    names = declared("exfem_srv.h")
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n


def test_host_library_exports_header_symbols():
    lib = C.CDLL(_native.HOST_LIB)
    for n in declared("exfem_host.h"):
        assert hasattr(lib, n), n


def test_argument_errors_need_no_device():
    from exfem.gpu import gpu_lib, default_opts
    L = gpu_lib()
    o = default_opts()
    assert o.precision == 0 and o.use_graph == 1 and o.reorder == 1
    h = C.c_void_p()
    assert L.exfem_gpu_create(None, None, C.byref(o), C.byref(h)) == EXFEM_E_ARG
    assert b"NULL" in L.exfem_gpu_last_error(None)
    m = Mesh()
    p = Problem()
    assert L.exfem_gpu_create(C.byref(m), C.byref(p), C.byref(o), C.byref(h)) == EXFEM_E_ARG
    bad = default_opts(block_threads=512)   # FP64 kernels take at most 256
    assert L.exfem_gpu_create(C.byref(m), C.byref(p), C.byref(bad), C.byref(h)) == EXFEM_E_ARG
    assert default_opts().index_bits == 0
    assert L.exfem_gpu_release_cached(-1) == EXFEM_E_ARG
    bad = default_opts(index_bits=32)   # 0 (automatic) or 64
    assert L.exfem_gpu_create(C.byref(m), C.byref(p), C.byref(bad), C.byref(h)) == EXFEM_E_ARG
    assert b"index_bits" in L.exfem_gpu_last_error(None)
    assert default_opts().drm_inline == 0 and default_opts().tune == 0 and default_opts().serial_launch == 0
    for field, bad_value in (("drm_inline", 2), ("tune", 2), ("serial_launch", -1)):
        bad = default_opts(**{field: bad_value})
        assert L.exfem_gpu_create(C.byref(m), C.byref(p), C.byref(bad), C.byref(h)) == EXFEM_E_ARG
        assert field.encode() in L.exfem_gpu_last_error(None)
    assert default_opts().wait_cycles == 0       # the library's default bound
    bad = default_opts(wait_cycles=-1)
    assert L.exfem_gpu_create(C.byref(m), C.byref(p), C.byref(bad), C.byref(h)) == EXFEM_E_ARG
    assert b"wait_cycles" in L.exfem_gpu_last_error(None)


def test_estimate_counts_rhs_padding():
    """exfem_gpu_estimate_bytes needs no device.  An FP32 context pads an odd
    right-hand-side count (13 -> 16) unless pad_rhs = 1, and its footprint
    estimate grows with the padding; FP64 contexts never pad."""
    from exfem import workloads
    from exfem.gpu import estimate_bytes
    waves = [("WAVEP" if i % 2 == 0 else "WAVESV", 2.0 * i) for i in range(13)]
    m = workloads.build("canyon", scale=0.1, steps=10, waves=waves)
    assert m.problem.nrhs == 13
    padded = estimate_bytes(m, precision=1)
    plain = estimate_bytes(m, precision=1, pad_rhs=1)
    assert padded > plain
    assert estimate_bytes(m, precision=0) == estimate_bytes(m, precision=0, pad_rhs=1)
    even = workloads.build("canyon", scale=0.1, steps=10, waves=waves[:12])
    assert estimate_bytes(even, precision=1) == estimate_bytes(even, precision=1, pad_rhs=1)


def test_server_defaults_keep_the_drm_pass_inline():
    """The server's default solver options run every request's DRM forces in
    its hanging/receiver pass (drm_inline = 1): with many requests stepping at
    once, a second stream per request measured slower.  A context made
    directly defaults to the second stream (drm_inline = 0)."""
    import ctypes as C

    from exfem.abi import SrvOpts
    from exfem.gpu import default_opts
    from exfem.serve import srv_lib
    o = SrvOpts()
    srv_lib().exfem_srv_default_opts(C.byref(o))
    assert o.solver.drm_inline == 1 and o.solver.precision == 1
    assert default_opts().drm_inline == 0
