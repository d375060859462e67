"""Continuous-batching solve server (C ABI dgx_server_*)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import call


def request(n: int, order: int, equation: int, ic: int, params=(), t_end: float = 0.1,
            lx: float = 1.0, ly: float = 1.0, jitter: float = 0.15, seed: int = 0,
            flux: int = _ffi.FLUX_LLF, precision: int = _ffi.FP32, gamma: float = 1.4,
            a=(1.0, 1.0), cfl: float = 0.7, dt: float = 0.0, keep_state: bool = False):
    r = _ffi.Request()
    r.n, r.lx, r.ly, r.jitter, r.seed = n, lx, ly, jitter, seed
    r.order, r.equation, r.flux, r.precision = order, equation, flux, precision
    r.gamma, r.ax, r.ay = gamma, float(a[0]), float(a[1])
    r.ic = ic
    for i, v in enumerate(params):
        r.params[i] = v
    r.t_end, r.cfl, r.dt, r.keep_state = t_end, cfl, dt, int(keep_state)
    return r


class Server:
    def __init__(self, budget_bytes: int, max_active: int = 512):
        h = C.c_void_p()
        call("dgx_server_create", int(budget_bytes), int(max_active), C.byref(h))
        self.h = h

    def submit(self, req) -> int:
        i = C.c_longlong()
        call("dgx_server_submit", self.h, C.byref(req), C.byref(i))
        return i.value

    def status(self, rid: int):
        st, lat = C.c_int(), C.c_double()
        rc = _ffi.lib().dgx_server_status(self.h, rid, C.byref(st), C.byref(lat))
        return st.value, lat.value, rc

    def result(self, rid: int, size: int = 0):
        out = np.zeros(max(size, 1))
        tot = np.zeros(4)
        steps, t = C.c_int(), C.c_double()
        call("dgx_server_result", self.h, rid,
             out.ctypes.data_as(C.POINTER(C.c_double)) if size else None, size,
             tot.ctypes.data_as(C.POINTER(C.c_double)), C.byref(steps), C.byref(t))
        return (out if size else None), tot, steps.value, t.value

    def cancel(self, rid: int) -> None:
        call("dgx_server_cancel", self.h, rid)

    def release(self, rid: int) -> None:
        call("dgx_server_release", self.h, rid)

    def wait_idle(self, timeout_s: float = 60.0) -> int:
        return _ffi.lib().dgx_server_wait_idle(self.h, float(timeout_s))

    def stats(self) -> dict:
        st = _ffi.ServerStats()
        call("dgx_server_get_stats", self.h, C.byref(st))
        return {k: getattr(st, k) for k, _ in _ffi.ServerStats._fields_}

    def set_steps_per_check(self, k: int) -> None:
        call("dgx_server_set_steps_per_check", self.h, int(k))

    def inject_stall(self, seconds: float) -> None:
        call("dgx_server_inject_stall", self.h, float(seconds))

    def close(self):
        if getattr(self, "h", None):
            _ffi.lib().dgx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
