"""Batches of independent solves advanced together (C ABI dgx_batch_*)."""
from __future__ import annotations

import ctypes as C

from . import _ffi
from ._ffi import call


class Batch:
    def __init__(self, solvers):
        self.solvers = list(solvers)          # keep the solvers alive
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = C.c_void_p()
        call("dgx_batch_create", arr, len(self.solvers), C.byref(h))
        self.h = h

    def step(self, stream: int = 0) -> None:
        call("dgx_batch_step", self.h, stream)

    def run(self, steps: int, stream: int = 0) -> None:
        call("dgx_batch_run", self.h, int(steps), stream)

    def autotune(self, reps: int = 3, stream: int = 0) -> None:
        call("dgx_batch_autotune", self.h, int(reps), stream)

    def info(self) -> dict:
        nc, ni = C.c_int(), C.c_int()
        dofs, lps = C.c_longlong(), C.c_longlong()
        call("dgx_batch_info", self.h, C.byref(nc), C.byref(ni), C.byref(dofs), C.byref(lps))
        return dict(classes=nc.value, items=ni.value, dofs=dofs.value, launches_per_step=lps.value)

    def class_options(self):
        out = []
        for k in range(self.info()["classes"]):
            v = [C.c_int() for _ in range(4)]
            call("dgx_batch_class_options", self.h, k, *[C.byref(x) for x in v])
            out.append(dict(order=v[0].value, equation=v[1].value, prefetch=v[2].value,
                            persistent=v[3].value))
        return out

    def set_fused(self, mode: int) -> None:
        """0: one launch per class and stage; 2 or 3: one fused launch per stage
        for every class (the kernel compiled for 2 or 3 CTAs per SM)."""
        call("dgx_batch_set_fused", self.h, int(mode))

    def fused(self) -> tuple[int, bool]:
        """(current fused mode, whether the batch allows the fused launch)"""
        m, a = C.c_int(), C.c_int()
        call("dgx_batch_get_fused", self.h, C.byref(m), C.byref(a))
        return m.value, bool(a.value)

    def launch_count(self) -> int:
        v = C.c_longlong()
        call("dgx_batch_launch_count", self.h, C.byref(v))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            _ffi.lib().dgx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
