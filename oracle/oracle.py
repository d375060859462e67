"""ctypes wrapper of the FP64 CPU oracle (oracle/dgx_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/ and ``__graft_entry__.smoke()``
(the oracle the CUDA path is tested against) and by the CPU-baseline leg of
``bench.py`` (timed as the CPU baseline); the product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_euler")

ADVECTION, EULER = 0, 1
CENTRAL, LLF = 0, 1
IC_GAUSSIAN, IC_POLY, IC_DENSITY_WAVE, IC_VORTEX, IC_CONSTANT = 0, 1, 2, 3, 4
IC_CYLINDER, IC_SUPERSONIC, IC_THREEPOINT, IC_LINEAR = 5, 6, 7, 8
RK4, RK2, FE = 0, 1, 2

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile liborc.so with the committed Makefile (gcc + OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "dgx_oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE, "lib"], check=True)
    return LIB_PATH


def env_reference_root() -> str | None:
    """The reference tree named by the environment variable DGX_REFERENCE_ROOT
    (the directory holding src/2d), or None when it is unset or absent."""
    root = os.environ.get("DGX_REFERENCE_ROOT", "")
    return root if root and os.path.isdir(root) else None


def install_ref(reference_root: str | None = None) -> bool:
    """Copy the reference's Euler sources the harnesses compile (unmodified) to
    baseline/_ref/src/2d, for machines without the reference tree.
    reference_root defaults to DGX_REFERENCE_ROOT; False without a tree."""
    reference_root = reference_root or env_reference_root()
    if not reference_root or not os.path.isdir(reference_root):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref-src", f"REF={reference_root}"], check=True)
    return True


def build_ref(reference_root: str | None = None) -> str | None:
    """Compile the reference's own CPU Euler loops, from the reference tree
    (reference_root, else DGX_REFERENCE_ROOT) or the installed copy under
    baseline/_ref; the binary path or None."""
    reference_root = reference_root or env_reference_root()
    cmd = ["make", "-s", "-C", HERE, "ref"] + ([f"REF={reference_root}"] if reference_root else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    return REF_BIN if r.returncode == 0 and os.path.exists(REF_BIN) else None


def time_ref_cpu(mesh, p: int, c0, dt: float, nsteps: int, procs: int = 1) -> list:
    """Wall seconds of `nsteps` RK4 steps of the reference's own CPU Euler loops
    (oracle/_ref/ref_euler, fixed dt) on `mesh` from c0, in `procs` processes
    run side by side (the reference's loops are serial); one figure per process."""
    ref_bin = build_ref()
    if ref_bin is None:
        raise RuntimeError("the reference's CPU loops are not built (no reference sources)")
    import tempfile
    E, S = mesh.num_elem, mesh.num_sides
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.bin")
        with open(fin, "wb") as f:
            np.array([E, S, p, nsteps, 0, 1, 0, 0], dtype=np.int32).tofile(f)
            np.array([dt], dtype=np.float64).tofile(f)
            for a in mesh.vertices():
                np.asarray(a, dtype=np.float64).tofile(f)
            for a in mesh.elem_sides():
                np.asarray(a, dtype=np.int32).tofile(f)
            for a in mesh.side_arrays():
                np.asarray(a, dtype=np.int32).tofile(f)
            np.asarray(c0, dtype=np.float64).tofile(f)
        outs = [os.path.join(td, f"out{k}.bin") for k in range(procs)]
        ps = [subprocess.Popen([ref_bin, fin, o], stdout=subprocess.DEVNULL) for o in outs]
        codes = [q.wait() for q in ps]
        if any(codes):
            raise RuntimeError(f"reference CPU loops failed: exit codes {codes}")
        secs = []
        for o in outs:
            with open(o, "rb") as f:
                f.seek(-8, os.SEEK_END)
                secs.append(float(np.frombuffer(f.read(8), dtype=np.float64)[0]))
    return secs


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = ([C.c_int, C.c_int] + [_dp] * 6 + [_ip] * 7
                                 + [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_double, C.c_int])
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_get_tables.argtypes = [C.c_int, _ip] + [_dp] * 10
        L.orc_geometry.argtypes = [C.c_void_p] + [_dp] * 9
        L.orc_min_diameter.argtypes = [C.c_void_p]
        L.orc_min_diameter.restype = C.c_double
        L.orc_project.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.orc_rhs.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_double]
        L.orc_max_lambda.argtypes = [C.c_void_p, _dp]
        L.orc_max_lambda.restype = C.c_double
        L.orc_cfl_dt.argtypes = [C.c_void_p, _dp, C.c_double]
        L.orc_cfl_dt.restype = C.c_double
        L.orc_rk4_step.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double]
        L.orc_step.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double]
        L.orc_set_integrator.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_limit_p1.argtypes = [C.c_void_p, _dp]
        L.orc_set_limiter.argtypes = [C.c_void_p, C.c_int]
        L.orc_run.argtypes = [C.c_void_p, _dp, C.c_int, C.c_double, C.c_double, C.c_double,
                              C.c_int, C.POINTER(C.c_double)]
        L.orc_totals.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_ic_eval.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double, _dp]
        L.orc_set_boundary.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


def num_modes(p: int) -> int:
    return (p + 1) * (p + 2) // 2


def tables(p: int) -> dict:
    L = lib()
    dims = np.zeros(3, dtype=np.int32)
    big = [np.zeros(2048) for _ in range(10)]
    if L.orc_get_tables(p, dims, *big):
        raise ValueError(f"unsupported order p={p}")
    np_, nq, nq1 = (int(x) for x in dims)
    r1, r2, w, s1, w1, phi, gx, gy, side, vert = big
    return dict(np=np_, nq=nq, nq1=nq1, r1=r1[:nq], r2=r2[:nq], w=w[:nq], s1=s1[:nq1],
                w1=w1[:nq1], phi=phi[:np_ * nq].reshape(np_, nq),
                gx=gx[:np_ * nq].reshape(np_, nq), gy=gy[:np_ * nq].reshape(np_, nq),
                side=side[:3 * np_ * nq1].reshape(3, np_, nq1), vert=vert[:3 * np_].reshape(np_, 3))


class Oracle:
    """FP64 restatement of the reference scheme on one mesh."""

    def __init__(self, mesh, p: int, equation: int = EULER, flux: int = LLF,
                 gamma: float = 1.4, a=(1.0, 1.0), ref_sqrtf: bool = False):
        L = lib()
        self.mesh = mesh
        self.p = p
        self.np = num_modes(p)
        self.nv = 4 if equation == EULER else 1
        self.E = mesh.num_elem
        self.S = mesh.num_sides
        self.equation = equation
        self.h = L.orc_create(mesh.num_elem, mesh.num_sides, *mesh.vertices(), *mesh.elem_sides(),
                              *mesh.side_arrays(), p, equation, flux, gamma, float(a[0]),
                              float(a[1]), int(ref_sqrtf))
        if not self.h:
            raise MemoryError("orc_create failed")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_destroy(h)
            self.h = None

    @property
    def shape(self):
        return (self.nv, self.np, self.E)

    def _state(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        if u.size != self.nv * self.np * self.E:
            raise ValueError("state has the wrong size")
        return u.reshape(self.shape)

    def geometry(self) -> dict:
        E, S = self.E, self.S
        out = dict(J=np.zeros(E), xr=np.zeros(E), yr=np.zeros(E), xs=np.zeros(E), ys=np.zeros(E),
                   len=np.zeros(S), nx=np.zeros(S), ny=np.zeros(S), diam=np.zeros(E))
        lib().orc_geometry(self.h, out["J"], out["xr"], out["yr"], out["xs"], out["ys"],
                           out["len"], out["nx"], out["ny"], out["diam"])
        return out

    def min_diameter(self) -> float:
        return lib().orc_min_diameter(self.h)

    def project(self, ic: int, params=()) -> np.ndarray:
        P = np.zeros(8)
        P[:len(params)] = params
        c = np.zeros(self.shape)
        lib().orc_project(self.h, ic, P, c)
        return c

    def rhs(self, u, dt: float = 1.0, t: float = 0.0) -> np.ndarray:
        u = self._state(u)
        k = np.zeros(self.shape)
        rc = lib().orc_rhs(self.h, u, k, dt, t)
        if rc:
            raise RuntimeError(f"orc_rhs failed ({rc})")
        return k

    def set_boundary(self, kind: int, ic: int = 0, params=()) -> None:
        """0 none, 1 free-stream state {rho, u, v, p}, 2 exact IC translated by a*t."""
        P = np.zeros(8)
        P[:len(params)] = params
        lib().orc_set_boundary(self.h, int(kind), int(ic), P)

    def set_integrator(self, integrator: int, reference_stage_time: bool = False) -> None:
        """RK4 (default), RK2 midpoint or FE; reference_stage_time selects the
        reference's stage-time arguments for time-dependent boundary data."""
        if lib().orc_set_integrator(self.h, int(integrator), int(bool(reference_stage_time))):
            raise ValueError(f"unknown integrator {integrator}")

    def limit(self, c) -> np.ndarray:
        """The p = 1 slope limiter applied to a copy of c."""
        c = self._state(c).copy()
        if lib().orc_limit_p1(self.h, c):
            raise ValueError("the limiter serves p = 1")
        return c

    def set_limiter(self, on: bool) -> None:
        """Apply the limiter to every stage's output state (p = 1)."""
        if lib().orc_set_limiter(self.h, int(bool(on))):
            raise ValueError("the limiter serves p = 1")

    def max_lambda(self, c) -> float:
        return lib().orc_max_lambda(self.h, self._state(c))

    def cfl_dt(self, c, cfl: float = 0.7) -> float:
        return lib().orc_cfl_dt(self.h, self._state(c), cfl)

    def step(self, c, dt: float, t: float = 0.0) -> np.ndarray:
        c = self._state(c).copy()
        rc = lib().orc_step(self.h, c, dt, t)
        if rc:
            raise RuntimeError(f"orc_step failed ({rc})")
        return c

    def run(self, c, t_end: float, dt: float | None = None, cfl: float = 0.7,
            max_steps: int = 0):
        """Advance to t_end (fixed dt, or the reference CFL rule when dt is
        None); returns (state, steps, t)."""
        c = self._state(c).copy()
        t = C.c_double(0.0)
        n = lib().orc_run(self.h, c, 0 if dt is not None else 1, dt or 0.0, cfl, t_end,
                          max_steps, C.byref(t))
        if n < 0:
            raise RuntimeError(f"orc_run failed ({n})")
        return c, n, t.value

    def totals(self, c) -> np.ndarray:
        out = np.zeros(4)
        lib().orc_totals(self.h, self._state(c), out)
        return out[:self.nv]


def ic_eval(ic: int, params, x: float, y: float, gamma: float = 1.4) -> np.ndarray:
    P = np.zeros(8)
    P[:len(params)] = params
    U = np.zeros(4)
    lib().orc_ic_eval(ic, P, gamma, float(x), float(y), U)
    return U


def rel_l2(a, b) -> np.ndarray:
    """Relative L2 error per variable (first axis) of a against b."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nv = a.shape[0]
    a = a.reshape(nv, -1)
    b = b.reshape(nv, -1)
    den = np.linalg.norm(b, axis=1)
    den = np.where(den == 0, 1.0, den)
    return np.linalg.norm(a - b, axis=1) / den
