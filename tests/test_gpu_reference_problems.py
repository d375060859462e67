"""Boundary sides and the reference's problem plug-ins pinned to the
reference's own CUDA solver on its own meshes.

oracle/ref_gpu_harness.cu is compiled with the reference's cylinder,
supersonic-vortex and three-point problem files (src/2d/conservation/euler/
cylinder/cylinder.cu, euler/supersonic/supersonic.cu,
euler/threepoint/threepoint.cu), whose hooks give the ghost states of
reflecting (-1), outflow (-2) and inflow (-3) sides (dispatched by
eval_left_right, src/2d/conservation/conserv_kernels.cu:657-679).  The meshes
are the reference's cylinder.pmsh and sv1.pmsh (tests/golden/
reference_meshes.npz); the three-point problem ships only its mesh
description (threepoint.geo), so its rectangle is triangulated here.  Both
sides start from the same FP64 coefficients and advance to the same end time
with the reference's CFL rule, with time_integrate_rk2 (the cylinder
problem's integrator, cylinder.cu:13, time_integrator.cu:466-614) or
time_integrate_rk4 (the supersonic and three-point problems').

The reference's hooks take square roots and powers in FP32 (sqrtf of the
radius in the radial reflections, powf in the supersonic state); the GPU path
does so with DGX_OPT_HOOK_MATH = DGX_HOOK_MATH_REFERENCE.  Its geometry and
sound speed also use float square roots (conserv_kernels.cu:346,364-371,
euler.cu:80), which the GPU path does not mimic: they move the LLF
dissipation at the cylinder's wall and at the three-point shock, where the
jumps are largest.  Measured on GB300 (max over variables): supersonic
2.3e-11 / 3e-14 (p = 1 / 3), cylinder 2.4e-9 .. 3.1e-9 (rho v, whose
free-stream value is 0; the other variables 2e-10 .. 5e-10) with the
reference hook arithmetic; 2.5e-8 .. 9.2e-8 with FP64 hooks; FP32 3.8e-7 ..
1.6e-6.  Three-point, p = 1 / 2: FP64 9.6e-9 .. 1.1e-8 / 2.3e-8 .. 2.4e-8,
FP32 5.7e-6 .. 7.0e-6 / 1.8e-5 .. 2.0e-5, all for rho v (the other variables
2.7e-10 .. 5.2e-9 and 9.5e-8 .. 2.4e-6).
Tolerances (relative L2 per conserved variable):
  FP64 path (reference hook arithmetic) vs the reference   <= 1e-8 (supersonic 1e-9,
                                                              three-point 1e-7)
  FP64 path (FP64 hook arithmetic) vs the reference        <= 1e-6
  FP32 path vs the reference                               <= 1e-5 (three-point rho v 5e-5)
"""
import os

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import from_triangles, read_pmsh
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_meshes.npz")
CYLINDER = (0.38,)          # MACH of cylinder.cu:11
SUPERSONIC = (2.25, 1.0125)  # MACH and the density constant of supersonic.cu:11,30
THREEPOINT = (0.25, 5.0)     # MACH and THETA (degrees) of threepoint.cu:14-15


@pytest.fixture(scope="module")
def ref_gpu():
    from oracle import ref_gpu
    if ref_gpu.build() is None:
        pytest.skip("the reference's CUDA sources are not at hand (make -C oracle ref-src)")
    return ref_gpu


def reference_mesh(name, tmp_path_factory):
    z = np.load(GOLDEN)
    p = tmp_path_factory.mktemp("meshes") / f"{name}.pmsh"
    p.write_bytes(z[f"{name}_pmsh"].tobytes())
    return read_pmsh(str(p))


def rel_l2(a, b):
    a = a.reshape(4, -1)
    b = b.reshape(4, -1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


CASES = [
    # (mesh, problem, initial-condition id, params, order, RK2?, CFL steps to the end time)
    ("cylinder", "cylinder", _ffi.IC_CYLINDER, CYLINDER, 1, True, 40.5),
    ("cylinder", "cylinder", _ffi.IC_CYLINDER, CYLINDER, 2, True, 30.5),
    ("cylinder", "cylinder", _ffi.IC_CYLINDER, CYLINDER, 2, False, 20.5),
    ("sv1", "supersonic", _ffi.IC_SUPERSONIC_VORTEX, SUPERSONIC, 1, False, 40.5),
    ("sv1", "supersonic", _ffi.IC_SUPERSONIC_VORTEX, SUPERSONIC, 3, False, 20.5),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[1]}-p{c[4]}-{'rk2' if c[5] else 'rk4'}" for c in CASES])
def test_problem_matches_reference_solver(case, ref_gpu, gpu, oracle_mod, tmp_path_factory):
    mesh_name, problem, ic, params, p, rk2, nsteps = case
    orc = oracle_mod
    m = reference_mesh(mesh_name, tmp_path_factory)
    m.check()
    o = orc.Oracle(m, p, orc.EULER, orc.LLF)
    c0 = o.project(ic, params)
    t_end = nsteps * o.cfl_dt(c0)
    ref = ref_gpu.run(m, p, c0, t_end, problem=problem, rk2=rk2)
    integrator = _ffi.RK2 if rk2 else _ffi.RK4
    errs = {}
    for precision, hook in ((_ffi.FP64, _ffi.HOOK_MATH_REFERENCE), (_ffi.FP64, _ffi.HOOK_MATH_DOUBLE),
                            (_ffi.FP32, _ffi.HOOK_MATH_REFERENCE)):
        sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision, integrator=integrator)
        sv.set_boundary(_ffi.BC_PROBLEM, ic, params)
        sv.set_option(_ffi.OPT_STAGE_TIME, _ffi.STAGE_TIME_REFERENCE)
        sv.set_option(_ffi.OPT_HOOK_MATH, hook)
        sv.set_state(c0)
        sv.set_dt(None, cfl=0.7)
        n, t = sv.run(t_end=t_end)
        assert n == ref["steps"], (n, ref["steps"])
        assert abs(t - t_end) <= 1e-12 * t_end
        errs[(precision, hook)] = rel_l2(sv.get_state(), ref["state"])
        sv.close()
    print(f"{problem} p={p} {'rk2' if rk2 else 'rk4'} steps={ref['steps']}: "
          + ", ".join(f"{'fp64' if k[0] == _ffi.FP64 else 'fp32'}/"
                      f"{'ref' if k[1] == _ffi.HOOK_MATH_REFERENCE else 'double'} {v.max():.2e}"
                      for k, v in errs.items()))
    assert errs[(_ffi.FP64, _ffi.HOOK_MATH_REFERENCE)].max() <= (1e-9 if problem == "supersonic" else 1e-8), errs
    assert errs[(_ffi.FP64, _ffi.HOOK_MATH_DOUBLE)].max() <= 1e-6, errs
    assert errs[(_ffi.FP32, _ffi.HOOK_MATH_REFERENCE)].max() <= 1e-5, errs


def run_both(m, p, ic, params, t_end_steps, problem, rk2, ref_gpu, orc):
    """The reference's solver and the GPU path in its three forms from the
    same FP64 coefficients to the same end time; relative L2 per form."""
    o = orc.Oracle(m, p, orc.EULER, orc.LLF)
    c0 = o.project(ic, params)
    t_end = t_end_steps * o.cfl_dt(c0)
    ref = ref_gpu.run(m, p, c0, t_end, problem=problem, rk2=rk2)
    errs = {}
    for precision, hook in ((_ffi.FP64, _ffi.HOOK_MATH_REFERENCE), (_ffi.FP64, _ffi.HOOK_MATH_DOUBLE),
                            (_ffi.FP32, _ffi.HOOK_MATH_REFERENCE)):
        sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision, integrator=_ffi.RK2 if rk2 else _ffi.RK4)
        sv.set_boundary(_ffi.BC_PROBLEM, ic, params)
        sv.set_option(_ffi.OPT_STAGE_TIME, _ffi.STAGE_TIME_REFERENCE)
        sv.set_option(_ffi.OPT_HOOK_MATH, hook)
        sv.set_state(c0)
        sv.set_dt(None, cfl=0.7)
        n, t = sv.run(t_end=t_end)
        assert n == ref["steps"], (n, ref["steps"])
        assert abs(t - t_end) <= 1e-12 * t_end
        errs[(precision, hook)] = rel_l2(sv.get_state(), ref["state"])
        sv.close()
    return errs, ref["steps"]


def threepoint_mesh(nx, ny, inflow, seed=5):
    """[0,1] x [0,0.5] in nx x ny cells, interior vertices jittered by 0.1 h,
    each cell split into two counter-clockwise triangles, numbered and sorted
    as the reference's converter does (from_triangles): the bottom line a
    reflecting wall (-1), the top line inflow (-3) with `inflow`, the rest
    outflow (-2)."""
    rng = np.random.default_rng(seed)
    xs, ys = np.linspace(0.0, 1.0, nx + 1), np.linspace(0.0, 0.5, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    inner = (X > 0) & (X < 1) & (Y > 0) & (Y < 0.5)
    X = X + inner * rng.uniform(-0.1, 0.1, X.shape) / nx
    Y = Y + inner * rng.uniform(-0.1, 0.1, Y.shape) * 0.5 / ny
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    v = lambda i, j: j * (nx + 1) + i
    tris = []
    for j in range(ny):
        for i in range(nx):
            tris.append((v(i, j), v(i + 1, j), v(i + 1, j + 1)))
            tris.append((v(i, j), v(i + 1, j + 1), v(i, j + 1)))

    def tag(a, b):
        (xa, ya), (xb, yb) = xy[a], xy[b]
        if ya == 0.0 and yb == 0.0:
            return -1
        if inflow and ya == 0.5 and yb == 0.5:
            return -3
        return -2
    return from_triangles(xy, tris, tag)


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("inflow", [False, True], ids=["geo-tags", "with-inflow"])
def test_threepoint_matches_reference_solver(p, inflow, ref_gpu, gpu, oracle_mod):
    """The three-point shock (threepoint.cu: an oblique shock state beside a
    resting gas, split along the ray at THETA, atan(x/y)) on the rectangle of
    its mesh description (threepoint.geo: [0,1] x [0,0.5], the bottom line
    physical 10000, a reflecting wall -1, the other three 20000, outflow -2),
    here a generated triangulation; with inflow the top side is -3 instead,
    which the problem file's U_inflow serves: the shock state left of the
    moving front x = M t cos(THETA) + tan(THETA), U0 right of it (itself the
    shock state left of the ray at THETA, the resting gas right of it).  The reference's reflecting hook
    tests sqrtf(m.n) > 0, i.e. the sign of m.n rounded to FP32."""
    m = threepoint_mesh(24, 12, inflow)
    errs, steps = run_both(m, p, _ffi.IC_THREEPOINT, THREEPOINT, 20.5, "threepoint", False, ref_gpu, oracle_mod)
    print(f"threepoint p={p} inflow={inflow} steps={steps}: "
          + ", ".join(f"{'fp64' if k[0] == _ffi.FP64 else 'fp32'}/"
                      f"{'ref' if k[1] == _ffi.HOOK_MATH_REFERENCE else 'double'} "
                      + " ".join(f"{x:.2e}" for x in v) for k, v in errs.items()))
    # measured on GB300: FP64 (either hook arithmetic) 2.7e-10 .. 2.4e-8, FP32
    # 9.5e-8 .. 2.0e-5; the largest are rho v, whose norm is a few per cent of
    # rho's (the shock state's rho v = gamma M sin(THETA) = 0.03, the resting
    # gas 0), so the same absolute differences weigh ~30x more relative to it
    assert errs[(_ffi.FP64, _ffi.HOOK_MATH_REFERENCE)].max() <= 1e-7, errs
    assert errs[(_ffi.FP64, _ffi.HOOK_MATH_DOUBLE)].max() <= 1e-6, errs
    fp32 = errs[(_ffi.FP32, _ffi.HOOK_MATH_REFERENCE)]
    assert fp32[[0, 1, 3]].max() <= 1e-5 and fp32[2] <= 5e-5, errs
