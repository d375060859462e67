"""Thin Python handles over the C ABI (used by the tests and bench.py).

``DeviceMesh`` uploads a :class:`dgcuda_gb300.mesh.Mesh`; ``Solver`` owns the
resident state of one solve.  States are numpy arrays of shape
``(num_vars, n_p, num_elem)`` in the reference layout ``c[n][i][e]``.
Streams are raw ``cudaStream_t`` values (an int, 0 = default stream).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import call

__all__ = ["DeviceMesh", "Solver", "tables", "num_modes"]


def num_modes(p: int) -> int:
    return (p + 1) * (p + 2) // 2


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def tables(p: int) -> dict:
    """The FP64 basis and quadrature tables the library uses for order p."""
    dims = (C.c_int * 3)()
    bufs = [np.zeros(2048) for _ in range(10)]
    call("dgx_tables", p, dims, *[_dp(b) for b in bufs])
    np_, nq, nq1 = dims[0], dims[1], dims[2]
    r1, r2, w, s1, w1, phi, gx, gy, side, vert = bufs
    return dict(np=np_, nq=nq, nq1=nq1, r1=r1[:nq], r2=r2[:nq], w=w[:nq], s1=s1[:nq1],
                w1=w1[:nq1], phi=phi[:np_ * nq].reshape(np_, nq),
                gx=gx[:np_ * nq].reshape(np_, nq), gy=gy[:np_ * nq].reshape(np_, nq),
                side=side[:3 * np_ * nq1].reshape(3, np_, nq1), vert=vert[:3 * np_].reshape(np_, 3))


class DeviceMesh:
    def __init__(self, mesh):
        self.mesh = mesh
        h = C.c_void_p()
        V = [np.ascontiguousarray(a, dtype=np.float64) for a in mesh.vertices()]
        I = [np.ascontiguousarray(a, dtype=np.int32) for a in mesh.elem_sides() + mesh.side_arrays()]
        call("dgx_mesh_create", mesh.num_elem, mesh.num_sides, *[_dp(a) for a in V],
             *[_ip(a) for a in I], C.byref(h))
        self.h = h
        self.num_elem = mesh.num_elem
        self.num_sides = mesh.num_sides

    @classmethod
    def periodic_square(cls, n: int, lx: float = 1.0, ly: float = 1.0, jitter: float = 0.0,
                        seed: int = 0) -> "DeviceMesh":
        """A structured periodic mesh built by the native generator (identical
        to dgcuda_gb300.mesh.periodic_square with the same arguments)."""
        self = cls.__new__(cls)
        self.mesh = None
        h = C.c_void_p()
        call("dgx_mesh_create_periodic_square", int(n), float(lx), float(ly), 0.0, 0.0,
             float(jitter), int(seed), C.byref(h))
        self.h = h
        self.num_elem = 2 * n * n
        self.num_sides = 3 * n * n
        return self

    def geometry(self) -> dict:
        E, S = self.num_elem, self.num_sides
        out = {k: np.zeros(E) for k in ("J", "xr", "yr", "xs", "ys", "diam")}
        out.update({k: np.zeros(S) for k in ("len", "nx", "ny")})
        call("dgx_mesh_geometry", self.h, *[_dp(out[k]) for k in
                                            ("J", "xr", "yr", "xs", "ys", "diam", "len", "nx", "ny")])
        return out

    def min_diameter(self) -> float:
        v = C.c_double()
        call("dgx_mesh_min_diameter", self.h, C.byref(v))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            _ffi.lib().dgx_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    def __init__(self, mesh, order: int, equation: int = _ffi.EULER, flux: int = _ffi.FLUX_LLF,
                 precision: int = _ffi.FP32, gamma: float = 1.4, a=(1.0, 1.0),
                 integrator: int = _ffi.RK4):
        self.dmesh = mesh if isinstance(mesh, DeviceMesh) else DeviceMesh(mesh)
        desc = _ffi.SolverDesc(order, equation, flux, precision, integrator, gamma, float(a[0]),
                               float(a[1]))
        h = C.c_void_p()
        call("dgx_solver_create", self.dmesh.h, C.byref(desc), C.byref(h))
        self.h = h
        self.order = order
        self.np = num_modes(order)
        self.nv = 4 if equation == _ffi.EULER else 1
        self.E = self.dmesh.num_elem
        self.precision = precision
        self.integrator = integrator

    @property
    def shape(self):
        return (self.nv, self.np, self.E)

    @property
    def size(self):
        return self.nv * self.np * self.E

    def close(self):
        if getattr(self, "h", None):
            _ffi.lib().dgx_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # state ---------------------------------------------------------------
    def set_state(self, c) -> None:
        c = np.ascontiguousarray(c, dtype=np.float64)
        if c.size != self.size:
            raise ValueError("state has the wrong size")
        call("dgx_set_state", self.h, _dp(c))

    def get_state(self) -> np.ndarray:
        c = np.zeros(self.shape)
        call("dgx_get_state", self.h, _dp(c))
        return c

    def set_state_f32(self, c: np.ndarray, stream: int = 0) -> None:
        call("dgx_set_state_f32", self.h, c.ctypes.data_as(C.POINTER(C.c_float)), stream)

    def get_state_f32(self, out: np.ndarray, stream: int = 0) -> None:
        call("dgx_get_state_f32", self.h, out.ctypes.data_as(C.POINTER(C.c_float)), stream)

    def state_ptr(self) -> int:
        p = C.c_void_p()
        call("dgx_state_device_ptr", self.h, C.byref(p))
        return p.value

    def project(self, ic: int, params=()) -> None:
        P = np.zeros(8)
        P[:len(params)] = params
        call("dgx_project_ic", self.h, ic, _dp(P))

    # hot path --------------------------------------------------------------
    def rhs_eval(self, u_ptr: int, k_ptr: int, dt: float = 1.0, t: float = 0.0,
                 stream: int = 0) -> None:
        call("dgx_rhs_eval", self.h, u_ptr, k_ptr, dt, t, stream)

    def set_dt(self, dt: float | None = None, cfl: float = 0.7) -> None:
        if dt is None:
            call("dgx_set_dt", self.h, _ffi.DT_CFL, 0.0, cfl)
        else:
            call("dgx_set_dt", self.h, _ffi.DT_FIXED, float(dt), cfl)

    def set_end_time(self, t_end: float) -> None:
        call("dgx_set_end_time", self.h, float(t_end))

    def rk_stage(self, stage: int, stream: int = 0) -> None:
        call("dgx_rk_stage", self.h, stage, stream)

    def step(self, stream: int = 0) -> None:
        call("dgx_step", self.h, stream)

    def run(self, t_end: float = 0.0, max_steps: int = 0, stream: int = 0):
        n = C.c_int()
        t = C.c_double()
        call("dgx_run", self.h, float(t_end), int(max_steps), C.byref(n), C.byref(t), stream)
        return n.value, t.value

    def time(self, stream: int = 0):
        t, dt = C.c_double(), C.c_double()
        call("dgx_time", self.h, C.byref(t), C.byref(dt), stream)
        return t.value, dt.value

    def reset_time(self, t: float = 0.0) -> None:
        call("dgx_reset_time", self.h, float(t))

    def totals(self, stream: int = 0) -> np.ndarray:
        out = np.zeros(4)
        call("dgx_conserved_totals", self.h, _dp(out), stream)
        return out[:self.nv]

    def max_wave_speed(self, stream: int = 0) -> float:
        v = C.c_double()
        call("dgx_max_wave_speed", self.h, C.byref(v), stream)
        return v.value

    def set_boundary(self, kind: int, ic: int = 0, params=()) -> None:
        P = np.zeros(8)
        P[:len(params)] = params
        call("dgx_solver_set_boundary", self.h, int(kind), int(ic), _dp(P))

    def limit(self, stream: int = 0) -> None:
        call("dgx_limit", self.h, stream)

    def state_change(self, prev_ptr: int, stream: int = 0) -> float:
        v = C.c_double()
        call("dgx_state_change", self.h, prev_ptr, C.byref(v), stream)
        return v.value

    def run_steady(self, tol: float, max_steps: int, stream: int = 0):
        n, chg = C.c_int(), C.c_double()
        call("dgx_run_steady", self.h, float(tol), int(max_steps), C.byref(n), C.byref(chg), stream)
        return n.value, chg.value

    def set_option(self, option: int, value: int) -> None:
        call("dgx_solver_set_option", self.h, int(option), int(value))

    def launch_count(self) -> int:
        v = C.c_longlong()
        call("dgx_launch_count", self.h, C.byref(v))
        return v.value
