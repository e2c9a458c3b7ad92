"""ctypes bindings of the C ABI (include/ubootgl_gb300.h).

The product path is the in-tree CUDA library; there is no CPU fallback.  If
the library is missing, importing the bindings raises.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libubootgl_gb300.so")

FIELDS = {"vx": 0, "vy": 1, "vx_back": 2, "vy_back": 3, "p": 4, "f": 5, "flag": 6,
          "vx_accum": 7, "vy_accum": 8, "vx_current": 9, "vy_current": 10}
BC = {"INFLOW": 0, "OUTFLOW": 1, "OUTFLOW_ZERO_PRESSURE": 2, "NOSLIP": 3}
SOLVE_FIXED, SOLVE_TOLERANCE = 0, 1
FP32, MIXED_FP16, MIXED_BF16 = 0, 1, 2

ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "ESTATE", -5: "ETIMEOUT", -6: "EBUSY"}


class UbgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "E?"), code, msg))
        self.code = code


class Options(C.Structure):
    _fields_ = [("solver_mode", C.c_int), ("vcycles", C.c_int), ("tol", C.c_float),
                ("max_vcycles", C.c_int), ("precision", C.c_int), ("use_graph", C.c_int),
                ("advect_bilinear", C.c_int)]


class ServeStats(C.Structure):
    _fields_ = [("sessions", C.c_int), ("queued", C.c_int), ("active", C.c_int),
                ("completed", C.c_longlong), ("rejected_sessions", C.c_longlong),
                ("cell_steps", C.c_longlong), ("device_bytes_used", C.c_size_t),
                ("busy_ms", C.c_double), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("max_ms", C.c_double), ("fused_steps", C.c_longlong),
                ("fused_member_steps", C.c_longlong), ("worker_fused_ms", C.c_double),
                ("worker_streams_ms", C.c_double), ("pending_sessions", C.c_int),
                ("admitted_from_queue", C.c_longlong)]


# name -> (restype, argtypes); every int-returning call is checked
_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_SIGS = {
    "ubg_last_error": (C.c_char_p, []),
    "ubg_device_info": (C.c_int, [C.c_char_p, C.c_size_t]),
    "ubg_create": (C.c_int, [_FP, C.c_int, C.c_int, C.c_float, C.c_float, C.POINTER(_P)]),
    "ubg_destroy": (C.c_int, [_P]),
    "ubg_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_P)]),
    "ubg_host_free": (C.c_int, [_P]),
    "ubg_default_options": (C.c_int, [C.POINTER(Options)]),
    "ubg_set_options": (C.c_int, [_P, C.POINTER(Options)]),
    "ubg_set_bcs": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int]),
    "ubg_step": (C.c_int, [_P, C.c_float]),
    "ubg_step_cfl": (C.c_int, [_P, C.c_float]),
    "ubg_last_dt": (C.c_int, [_P, _FP]),
    "ubg_solver_stats": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "ubg_scatter_accum": (C.c_int, [_P, C.c_int, _FP, _FP]),
    "ubg_sample_velocity": (C.c_int, [_P, C.c_int, _FP, _FP]),
    "ubg_set_grids": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int), _FP]),
    "ubg_shift_map": (C.c_int, [_P, _FP]),
    "ubg_snapshot_bytes": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "ubg_snapshot": (C.c_int, [_P, C.c_void_p]),
    "ubg_restore": (C.c_int, [_P, C.c_void_p]),
    "ubg_autotune": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "ubg_batch_create": (C.c_int, [C.c_int, C.POINTER(_P), C.POINTER(_P)]),
    "ubg_batch_destroy": (C.c_int, [_P]),
    "ubg_batch_step": (C.c_int, [_P, _FP, C.c_float]),
    "ubg_batch_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "ubg_batch_sync": (C.c_int, [_P]),
    "ubg_io_upload_async": (C.c_int, [_P, _FP, _FP]),
    "ubg_io_download_async": (C.c_int, [_P, _FP, _FP]),
    "ubg_io_wait": (C.c_int, [_P]),
    "ubg_selftest_div": (C.c_int, [_FP, C.c_int, C.c_float, C.POINTER(C.c_uint)]),
    "ubg_device_bytes": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_size_t)]),
    "ubg_sim_device_bytes": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "ubg_server_create": (C.c_int, [C.c_size_t, C.c_int, C.POINTER(_P)]),
    "ubg_server_destroy": (C.c_int, [_P]),
    "ubg_server_set_mode": (C.c_int, [_P, C.c_int]),
    "ubg_server_set_fuse_cells": (C.c_int, [_P, C.c_longlong]),
    "ubg_server_set_admission": (C.c_int, [_P, C.c_int]),
    "ubg_server_open": (C.c_int, [_P, _FP, C.c_int, C.c_int, C.c_float, C.c_float, _FP, _FP,
                                  C.POINTER(Options), C.POINTER(C.c_int)]),
    "ubg_server_close": (C.c_int, [_P, C.c_int]),
    "ubg_server_submit": (C.c_int, [_P, C.c_int, C.c_int, C.c_float, C.POINTER(C.c_uint64)]),
    "ubg_server_wait": (C.c_int, [_P, C.c_uint64, C.POINTER(C.c_double)]),
    "ubg_server_drain": (C.c_int, [_P]),
    "ubg_server_session_sim": (C.c_int, [_P, C.c_int, C.POINTER(_P)]),
    "ubg_server_stats": (C.c_int, [_P, C.POINTER(ServeStats)]),
    "ubg_apply_accumulated_velocity": (C.c_int, [_P]),
    "ubg_diffuse": (C.c_int, [_P, C.c_float]),
    "ubg_advect": (C.c_int, [_P, C.c_float]),
    "ubg_set_vbcs": (C.c_int, [_P]),
    "ubg_set_pbc": (C.c_int, [_P]),
    "ubg_project": (C.c_int, [_P, C.c_float]),
    "ubg_add_sink": (C.c_int, [_P, C.c_float, C.c_float, C.c_float]),
    "ubg_upload": (C.c_int, [_P, C.c_int, _FP]),
    "ubg_download": (C.c_int, [_P, C.c_int, _FP]),
    "ubg_mg_levels": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "ubg_mg_level_flag": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), _FP]),
    "ubg_mg_solve_sim": (C.c_int, [_P, C.c_int]),
    "ubg_field_device": (C.c_int, [_P, C.c_int, C.POINTER(_P), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ubg_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "ubg_sync": (C.c_int, [_P]),
    "ubg_profile_enable": (C.c_int, [_P, C.c_int]),
    "ubg_profile_read": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                   C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "ubg_profile_class": (C.c_int, [_P, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                    C.POINTER(C.c_int)]),
    "ubg_profile_reset": (C.c_int, [_P]),
    "ubg_velocity_texture": (C.c_int, [_P, _FP, _FP]),
    "ubg_tracers_create": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(_P)]),
    "ubg_tracers_destroy": (C.c_int, [_P]),
    "ubg_tracers_upload": (C.c_int, [_P, _FP, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), _FP]),
    "ubg_tracers_download": (C.c_int, [_P, _FP, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                       _FP]),
    "ubg_tracers_step": (C.c_int, [_P, C.c_float, C.c_uint32]),
    "ubg_mg_create": (C.c_int, [C.c_int, C.c_int, _FP, C.POINTER(_P)]),
    "ubg_mg_destroy": (C.c_int, [_P]),
    "ubg_mg_update_fields": (C.c_int, [_P, _FP]),
    "ubg_mg_solve": (C.c_int, [_P, _FP, _FP, _FP, C.c_float, C.c_int]),
    "ubg_mg_solve_device": (C.c_int, [_P, _P, C.c_int, _P, C.c_int, _P, C.c_int, C.c_float,
                                      C.c_int, _P]),
    "ubg_mg_solve_noalloc": (C.c_int, [_P, C.c_int, _P, C.c_int, _P, C.c_int, C.c_int, C.c_int,
                                       C.c_float, C.c_int, _P]),
    "ubg_rbgs": (C.c_int, [_FP, _FP, _FP, C.c_int, C.c_int, C.c_float, C.c_float]),
    "ubg_residual": (C.c_int, [_FP, _FP, _FP, _FP, C.c_int, C.c_int, C.c_float,
                               C.POINTER(C.c_double)]),
}

_lib = None


def declared_symbols():
    """Function names declared in include/*.h (parsed, for the export test)."""
    import re
    inc = os.path.join(os.path.dirname(_HERE), "include")
    names = []
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            txt = open(os.path.join(inc, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"\b(ubg_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def load(path=None):
    """Load the library and bind every function; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("ubootgl_gb300 CUDA library not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def extra_sig(name, res, args):
    lib = load()
    fn = getattr(lib, name)
    fn.restype = res
    fn.argtypes = args
    return fn


def check(code):
    if code != 0:
        msg = load().ubg_last_error().decode(errors="replace")
        raise UbgError(code, msg)
    return code


def fptr(a):
    return a.ctypes.data_as(_FP)


class PinnedArray:
    """A numpy float32 array in page-locked host memory (ubg_host_alloc)."""

    def __init__(self, shape):
        import numpy as np
        lib = load()
        n = int(np.prod(shape)) * 4
        self._p = C.c_void_p()
        check(lib.ubg_host_alloc(n, C.byref(self._p)))
        buf = (C.c_float * int(np.prod(shape))).from_address(self._p.value)
        self.array = np.ctypeslib.as_array(buf).reshape(shape)

    def __del__(self):
        if getattr(self, "_p", None) and self._p.value:
            try:
                load().ubg_host_free(self._p)
            except Exception:
                pass
            self._p = None
