"""ctypes mirror of include/exfem_gpu.h and include/exfem_host.h."""
from __future__ import annotations

import ctypes as C

EXFEM_OK = 0
EXFEM_E_ARG = -1
EXFEM_E_MESH = -2
EXFEM_E_NOMEM = -3
EXFEM_E_UNSUPPORTED = -4
EXFEM_E_CUDA = -5
EXFEM_E_NAN = -6
EXFEM_E_TIMEOUT = -7
EXFEM_E_STATE = -8

ERROR_NAMES = {
    EXFEM_E_ARG: "EXFEM_E_ARG", EXFEM_E_MESH: "EXFEM_E_MESH", EXFEM_E_NOMEM: "EXFEM_E_NOMEM",
    EXFEM_E_UNSUPPORTED: "EXFEM_E_UNSUPPORTED", EXFEM_E_CUDA: "EXFEM_E_CUDA",
    EXFEM_E_NAN: "EXFEM_E_NAN", EXFEM_E_TIMEOUT: "EXFEM_E_TIMEOUT", EXFEM_E_STATE: "EXFEM_E_STATE",
}

EXFEM_WAVE_P = 1
EXFEM_WAVE_SV = 2

EXFEM_POINT_FORCE = 1
EXFEM_POINT_DISP = 2

EXFEM_FP64 = 0
EXFEM_FP32_KAHAN = 1

EXFEM_VARIANT_REFERENCE_ORDER = 0
EXFEM_VARIANT_CLOSED_FORM = 1

EXFEM_HANG_HALF = 0
EXFEM_HANG_LITERAL = 1


class ExfemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERROR_NAMES.get(code, "?"), code, msg))
        self.code = code


class Wave(C.Structure):
    _fields_ = [("kind", C.c_int), ("amp", C.c_double), ("angle", C.c_double),
                ("freq", C.c_double), ("t0", C.c_double)]


class Mesh(C.Structure):
    _fields_ = [("nelems", C.c_int), ("nnodes", C.c_int),
                ("eptr", C.POINTER(C.c_int)), ("eind", C.POINTER(C.c_int)),
                ("ediv", C.POINTER(C.c_ubyte)), ("nodes", C.POINTER(C.c_double)),
                ("ematprop", C.POINTER(C.c_int))]


class Problem(C.Structure):
    _fields_ = [("nmat", C.c_int), ("matconst", C.POINTER(C.c_double)),
                ("absorbing", C.POINTER(C.c_int)),
                ("nhanging", C.c_int), ("hanging", C.POINTER(C.c_int)),
                ("nseismic", C.c_int), ("seismic", C.POINTER(C.c_int)),
                ("deltat", C.c_double), ("nsteps", C.c_int), ("io_interval", C.c_int),
                ("worigin", C.c_double * 2), ("wbox", C.c_double * 3),
                ("walpha", C.c_double), ("wbeta", C.c_double),
                ("nrhs", C.c_int), ("waves", C.POINTER(Wave)),
                ("nrecv", C.c_int), ("recv_xy", C.POINTER(C.c_double)),
                ("recv_elem", C.POINTER(C.c_int)),
                ("point_kind", C.c_int), ("npoint", C.c_int), ("point_nodes", C.POINTER(C.c_int)),
                ("point_amp", C.c_double), ("point_sigma", C.c_double), ("point_t0", C.c_double)]


class Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("use_graph", C.c_int),
                ("graph_steps", C.c_int), ("block_threads", C.c_int),
                ("rhs_per_thread", C.c_int), ("reorder", C.c_int), ("check_every", C.c_int),
                ("variant", C.c_int), ("index_bits", C.c_int), ("pad_rhs", C.c_int),
                ("wait_cycles", C.c_int), ("tune", C.c_int), ("drm_inline", C.c_int),
                ("serial_launch", C.c_int)]


class ModelInfo(C.Structure):
    _fields_ = [("width", C.c_double), ("height", C.c_double), ("duration", C.c_double),
                ("inttime", C.c_double), ("chper", C.c_double), ("nperlen", C.c_double),
                ("sperlen", C.c_double), ("blength", C.c_double), ("mlength", C.c_double),
                ("totcols", C.c_int), ("totrows", C.c_int), ("wrows", C.c_int), ("wcols", C.c_int),
                ("nmat_base", C.c_int), ("nmat", C.c_int), ("nelems", C.c_int), ("nnodes", C.c_int),
                ("nhanging", C.c_int), ("nseismic", C.c_int), ("nrecv", C.c_int), ("nrhs", C.c_int),
                ("nsteps", C.c_int), ("io_interval", C.c_int), ("deltat", C.c_double),
                ("nlevels", C.c_int), ("min_h", C.c_double), ("max_h", C.c_double)]


class SrvOpts(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_active", C.c_int), ("chunk_steps", C.c_int),
                ("preparers", C.c_int), ("max_bypass", C.c_int), ("solver", Opts)]


class SrvResult(C.Structure):
    _fields_ = [("id", C.c_longlong), ("status", C.c_int), ("nsteps", C.c_int), ("nelems", C.c_int),
                ("nrhs", C.c_int), ("nrecv", C.c_int), ("nsave", C.c_int), ("device_bytes", C.c_size_t),
                ("reserved_bytes", C.c_size_t),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_ready", C.c_double),
                ("t_done", C.c_double), ("t_meshed", C.c_double)]


SRV_SYMBOLS = {
    "exfem_srv_default_opts": (None, [C.POINTER(SrvOpts)]),
    "exfem_srv_open": (C.c_int, [C.POINTER(SrvOpts), C.POINTER(C.c_void_p)]),
    "exfem_srv_submit": (C.c_int, [C.c_void_p, C.POINTER(Mesh), C.POINTER(Problem), C.c_int,
                                   C.POINTER(C.c_longlong)]),
    "exfem_srv_submit_deck": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_longlong)]),
    "exfem_srv_poll": (C.c_int, [C.c_void_p, C.POINTER(SrvResult), C.c_int, C.c_int]),
    "exfem_srv_fetch": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_double), C.c_size_t]),
    "exfem_srv_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_longlong), C.POINTER(C.c_size_t), C.POINTER(C.c_int)]),
    "exfem_srv_last_error": (C.c_char_p, [C.c_void_p]),
    "exfem_srv_close": (None, [C.c_void_p]),
}

GPU_SYMBOLS = {
    "exfem_gpu_default_opts": (None, [C.POINTER(Opts)]),
    "exfem_gpu_create": (C.c_int, [C.POINTER(Mesh), C.POINTER(Problem), C.POINTER(Opts),
                                   C.POINTER(C.c_void_p)]),
    "exfem_gpu_init_explicit": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "exfem_gpu_run": (C.c_int, [C.c_void_p, C.c_int]),
    "exfem_gpu_sync": (C.c_int, [C.c_void_p]),
    "exfem_gpu_query": (C.c_int, [C.c_void_p]),
    "exfem_gpu_get_u": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t]),
    "exfem_gpu_get_seismograms": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t,
                                            C.POINTER(C.c_int)]),
    "exfem_gpu_sample_points": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double),
                                          C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "exfem_gpu_run_timed": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "exfem_gpu_profile_kernels": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                            C.POINTER(C.c_char_p), C.c_int]),
    "exfem_gpu_autotune": (C.c_int, [C.POINTER(Mesh), C.POINTER(Problem), C.POINTER(Opts), C.c_int,
                                     C.POINTER(C.c_double)]),
    "exfem_gpu_step_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "exfem_gpu_steps_done": (C.c_int, [C.c_void_p]),
    "exfem_gpu_launch_count": (C.c_longlong, [C.c_void_p]),
    "exfem_gpu_device_bytes": (C.c_size_t, [C.c_void_p]),
    "exfem_gpu_copy_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]),
    "exfem_gpu_release_cached": (C.c_int, [C.c_int]),
    "exfem_gpu_estimate_bytes": (C.c_size_t, [C.POINTER(Mesh), C.POINTER(Problem), C.POINTER(Opts)]),
    "exfem_gpu_last_error": (C.c_char_p, [C.c_void_p]),
    "exfem_gpu_destroy": (None, [C.c_void_p]),
}

class Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("origin", C.c_double * 2), ("space", C.c_double),
                ("npoints", C.c_int), ("points", C.POINTER(C.c_double)), ("elem", C.POINTER(C.c_int)),
                ("material", C.POINTER(C.c_double)), ("ncells", C.c_int), ("eptr", C.POINTER(C.c_int)),
                ("eind", C.POINTER(C.c_int)), ("nfound", C.c_int)]


HOST_SYMBOLS = {
    "exfem_model_build": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "exfem_model_error": (C.c_char_p, []),
    "exfem_model_views": (None, [C.c_void_p, C.POINTER(Mesh), C.POINTER(Problem)]),
    "exfem_model_get_info": (None, [C.c_void_p, C.POINTER(ModelInfo)]),
    "exfem_model_set_nsteps": (C.c_int, [C.c_void_p, C.c_int]),
    "exfem_model_save_mesh": (C.c_int, [C.c_void_p, C.c_char_p]),
    "exfem_write_mass": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_double)]),
    "exfem_write_step": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "exfem_write_sheet": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_double), C.c_int,
                                    C.POINTER(C.c_double), C.c_double]),
    "exfem_model_grid": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.POINTER(C.POINTER(Grid))]),
    "exfem_grid_free": (None, [C.POINTER(Grid)]),
    "exfem_write_vtu": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int,
                                  C.POINTER(C.c_double), C.c_char_p, C.POINTER(C.c_double)]),
    "exfem_model_free": (None, [C.c_void_p]),
}


def bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
