"""ctypes bindings of the C ABI in include/dgx.h (libdgx.so).

There is no fallback: if the native library is missing or does not load, every
entry point raises.  Build it with ``python -m dgcuda_gb300.build``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libdgx.so")

OK = 0
ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_UNSUPPORTED = -1, -2, -3, -4
ERR_NONFINITE, ERR_BUSY, ERR_NOT_FOUND, ERR_TIMEOUT = -5, -6, -7, -8

ADVECTION, EULER = 0, 1
FLUX_CENTRAL, FLUX_LLF = 0, 1
FP32, FP32_BF16X3, FP64, FP32_COMP = 0, 1, 2, 3
RK4, RK2, FE = 0, 1, 2
DT_FIXED, DT_CFL = 0, 1
OPT_PREFETCH, OPT_STAGE_TIME, OPT_LIMITER, OPT_HOOK_MATH = 1, 2, 3, 4
HOOK_MATH_DOUBLE, HOOK_MATH_REFERENCE = 0, 1
STAGE_TIME_EXACT, STAGE_TIME_REFERENCE = 0, 1
BC_NONE, BC_FREESTREAM, BC_EXACT, BC_PROBLEM = 0, 1, 2, 3
IC_GAUSSIAN, IC_POLY, IC_DENSITY_WAVE, IC_VORTEX, IC_CONSTANT = 0, 1, 2, 3, 4
IC_CYLINDER, IC_SUPERSONIC_VORTEX, IC_THREEPOINT, IC_LINEAR = 5, 6, 7, 8


class DgxError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {message} (status {status})")
        self.status = status


class SolverDesc(C.Structure):
    _fields_ = [("order", C.c_int), ("equation", C.c_int), ("flux", C.c_int),
                ("precision", C.c_int), ("integrator", C.c_int), ("gamma", C.c_double),
                ("ax", C.c_double), ("ay", C.c_double)]


class Request(C.Structure):
    _fields_ = [("n", C.c_int), ("lx", C.c_double), ("ly", C.c_double), ("jitter", C.c_double),
                ("seed", C.c_ulonglong), ("order", C.c_int), ("equation", C.c_int),
                ("flux", C.c_int), ("precision", C.c_int), ("gamma", C.c_double),
                ("ax", C.c_double), ("ay", C.c_double), ("ic", C.c_int),
                ("params", C.c_double * 8), ("t_end", C.c_double), ("cfl", C.c_double),
                ("dt", C.c_double), ("keep_state", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("active", C.c_longlong), ("queued", C.c_longlong), ("repacks", C.c_longlong),
                ("steps", C.c_longlong), ("dof_updates", C.c_double),
                ("busy_seconds", C.c_double), ("p50_latency_s", C.c_double),
                ("p99_latency_s", C.c_double), ("max_latency_s", C.c_double),
                ("device_bytes_in_use", C.c_size_t), ("admit_seconds", C.c_double),
                ("repack_seconds", C.c_double), ("retire_seconds", C.c_double),
                ("idle_seconds", C.c_double), ("pool_hits", C.c_longlong),
                ("pool_misses", C.c_longlong), ("cached_meshes", C.c_longlong)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = 0, 1, 2, 3, 4

# name -> (restype, argtypes); restype None means int status
_vp, _dp, _ip, _i, _d, _sz = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int, C.c_double, C.c_size_t
SIGNATURES = {
    "dgx_version": (C.c_int, []),
    "dgx_status_string": (C.c_char_p, [_i]),
    "dgx_last_error": (C.c_char_p, []),
    "dgx_tables": (None, [_i, _ip] + [_dp] * 10),
    "dgx_mesh_create": (None, [_i, _i] + [_dp] * 6 + [_ip] * 7 + [C.POINTER(_vp)]),
    "dgx_mesh_destroy": (None, [_vp]),
    "dgx_pmsh_info": (None, [C.c_char_p, _ip, _ip]),
    "dgx_pmsh_read": (None, [C.c_char_p, _dp, _ip, _ip]),
    "dgx_pmsh_write": (None, [C.c_char_p, _i, _i, _dp, _ip, _ip]),
    "dgx_mesh_create_from_pmsh": (None, [C.c_char_p, C.POINTER(_vp)]),
    "dgx_write_vertex_values": (None, [_vp, C.c_char_p]),
    "dgx_periodic_square_arrays": (None, [_i, _d, _d, _d, _d, _d, C.c_ulonglong, _dp, _ip, _ip]),
    "dgx_mesh_create_periodic_square": (None, [_i, _d, _d, _d, _d, _d, C.c_ulonglong, C.POINTER(_vp)]),
    "dgx_mesh_geometry": (None, [_vp] + [_dp] * 9),
    "dgx_mesh_min_diameter": (None, [_vp, _dp]),
    "dgx_mesh_info": (None, [_vp, _ip, _ip, _ip]),
    "dgx_solver_create": (None, [_vp, C.POINTER(SolverDesc), C.POINTER(_vp)]),
    "dgx_solver_destroy": (None, [_vp]),
    "dgx_solver_info": (None, [_vp, _ip, _ip, C.POINTER(_sz), C.POINTER(_sz)]),
    "dgx_set_state": (None, [_vp, _dp]),
    "dgx_get_state": (None, [_vp, _dp]),
    "dgx_set_state_f32": (None, [_vp, C.POINTER(C.c_float), _vp]),
    "dgx_get_state_f32": (None, [_vp, C.POINTER(C.c_float), _vp]),
    "dgx_state_device_ptr": (None, [_vp, C.POINTER(_vp)]),
    "dgx_project_ic": (None, [_vp, _i, _dp]),
    "dgx_rhs_eval": (None, [_vp, _vp, _vp, _d, _d, _vp]),
    "dgx_set_dt": (None, [_vp, _i, _d, _d]),
    "dgx_set_end_time": (None, [_vp, _d]),
    "dgx_rk_stage": (None, [_vp, _i, _vp]),
    "dgx_step": (None, [_vp, _vp]),
    "dgx_run": (None, [_vp, _d, _i, _ip, _dp, _vp]),
    "dgx_time": (None, [_vp, _dp, _dp, _vp]),
    "dgx_reset_time": (None, [_vp, _d]),
    "dgx_conserved_totals": (None, [_vp, _dp, _vp]),
    "dgx_conserved_totals_static": (None, [_vp, _vp, _vp, _vp]),
    "dgx_max_wave_speed": (None, [_vp, _dp, _vp]),
    "dgx_launch_count": (None, [_vp, C.POINTER(C.c_longlong)]),
    "dgx_tc_selftest": (None, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), _vp]),
    "dgx_limit": (None, [_vp, _vp]),
    "dgx_state_change": (None, [_vp, _vp, _dp, _vp]),
    "dgx_run_steady": (None, [_vp, _d, _i, _ip, _dp, _vp]),
    "dgx_solver_set_option": (None, [_vp, _i, _i]),
    "dgx_solver_set_boundary": (None, [_vp, _i, _i, _dp]),
    "dgx_batch_create": (None, [C.POINTER(_vp), _i, C.POINTER(_vp)]),
    "dgx_batch_destroy": (None, [_vp]),
    "dgx_batch_step": (None, [_vp, _vp]),
    "dgx_batch_run": (None, [_vp, _i, _vp]),
    "dgx_batch_autotune": (None, [_vp, _i, _vp]),
    "dgx_batch_info": (None, [_vp, _ip, _ip, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "dgx_batch_class_options": (None, [_vp, _i, _ip, _ip, _ip, _ip]),
    "dgx_batch_launch_count": (None, [_vp, C.POINTER(C.c_longlong)]),
    "dgx_batch_progress": (None, [_vp, _dp, _dp, C.POINTER(C.c_uint), C.POINTER(C.c_longlong), _vp]),
    "dgx_batch_set_options": (None, [_vp, _i, _i, _i]),
    "dgx_batch_set_fused": (None, [_vp, _i]),
    "dgx_batch_get_fused": (None, [_vp, _vp, _vp]),
    "dgx_server_create": (None, [_sz, _i, C.POINTER(_vp)]),
    "dgx_server_submit": (None, [_vp, C.POINTER(Request), C.POINTER(C.c_longlong)]),
    "dgx_server_status": (None, [_vp, C.c_longlong, _ip, _dp]),
    "dgx_server_result": (None, [_vp, C.c_longlong, _dp, _sz, _dp, _ip, _dp]),
    "dgx_server_cancel": (None, [_vp, C.c_longlong]),
    "dgx_server_release": (None, [_vp, C.c_longlong]),
    "dgx_server_wait_idle": (None, [_vp, _d]),
    "dgx_server_get_stats": (None, [_vp, C.POINTER(ServerStats)]),
    "dgx_server_set_steps_per_check": (None, [_vp, _i]),
    "dgx_server_inject_stall": (None, [_vp, _d]),
    "dgx_server_destroy": (None, [_vp]),
}

_lib = None
_lock = threading.Lock()


def lib():
    """Load libdgx.so (raises if it is missing: there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"native library {LIB_PATH} is missing; run "
                                  "`python -m dgcuda_gb300.build`")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res if res is not None else C.c_int
                fn.argtypes = args
            _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != OK:
        L = lib()
        msg = (L.dgx_last_error() or b"").decode(errors="replace")
        if not msg:
            msg = (L.dgx_status_string(status) or b"").decode()
        raise DgxError(status, where, msg)


def call(name: str, *args):
    check(getattr(lib(), name)(*args), name)


def exported_symbols():
    return list(SIGNATURES)
