"""Parity with the reference's own CUDA solvers, rebuilt for sm_103a and run on
the same GPU (oracle/ref_gpu_harness.cu drives the reference's Euler
time_integrate_rk4, src/2d/conservation/time_integrator.cu:221-434, and its
advection time_integrate_rk4, src/2d/time_integrator.cu:89-315, unchanged).

Advection: the reference hard-wires a = (1,1) and the central flux
(src/2d/2dadvec/2dadvec_kernels.cu:150-164); both sides take the same number of
steps of the same fixed dt from the same FP64 coefficients.  Its side lengths
and normals also use float square roots.  On meshes with boundary sides (-1)
the reference takes the exact data of its problem, x - 2t + y
(boundary_exact, 2dadvec_kernels.cu:184-186) at t = the step's start
(src/2d/time_integrator.cu:144-145) in every stage; the GPU path takes
DGX_BC_EXACT with DGX_IC_LINEAR {0, 1, 1} and the reference's stage times.
Tolerances: FP64 path <= 1e-9, FP32 path <= 1e-5.

Euler:

Both sides start from the same FP64 coefficients and advance to the same end
time with the same CFL rule (dt = 0.7 min_d / max lambda / (2p+1), the last step
clipped) and take the same number of steps.  The reference evaluates side
lengths, normals, inscribed radii and the sound speed with float square roots
(conserv_kernels.cu:346,364-371, euler.cu:80): its dt and LLF dissipation differ
from exact FP64 by ~1e-7 relative, which moves the states by far less (the end
time is the same; the dissipation acts on small jumps).  Measured on GB300: FP64
path 2e-13..7e-11, FP32 path 3e-7..2e-6.  Tolerances (relative L2 per conserved
variable):
  FP64 path vs the reference          <= 1e-9
  FP32 path vs the reference          <= 1e-5   (the FP32 path's accuracy bound)
"""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import from_triangles, periodic_square
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

VORTEX = (5.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0)
WAVE = (0.2, 1.0, 1.0, 1.0, 1.0)


@pytest.fixture(scope="module")
def ref_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from oracle import ref_gpu
    if ref_gpu.build() is None:
        pytest.skip("the reference's CUDA sources are not at hand (make -C oracle ref-src)")
    return ref_gpu


def rel_l2(a, b):
    a = a.reshape(4, -1)
    b = b.reshape(4, -1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def ours(mesh, p, precision, c0, t_end, integrator=_ffi.RK4):
    sv = Solver(mesh, p, _ffi.EULER, _ffi.FLUX_LLF, precision, integrator=integrator)
    sv.set_state(c0)
    sv.set_dt(None, cfl=0.7)
    n, t = sv.run(t_end=t_end)
    out = sv.get_state()
    sv.close()
    return out, n, t


@pytest.mark.parametrize("case", [
    ("vortex", 16, 10.0, 2, _ffi.IC_VORTEX, VORTEX, 0.25),
    ("density wave", 12, 1.0, 3, _ffi.IC_DENSITY_WAVE, WAVE, 0.02),
    ("vortex p=1", 20, 10.0, 1, _ffi.IC_VORTEX, VORTEX, 0.2),
    ("vortex p=4", 8, 10.0, 4, _ffi.IC_VORTEX, VORTEX, 0.3),
], ids=lambda c: c[0])
def test_paths_match_reference_gpu_solver(ref_gpu, case):
    _, n, L, p, ic, params, t_end = case
    mesh = periodic_square(n, lx=L, ly=L, jitter=0.15, seed=11 + n)
    init = Solver(mesh, p, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP64)
    init.project(ic, params)
    c0 = init.get_state()
    init.close()
    ref = ref_gpu.run(mesh, p, c0, t_end)
    assert ref["steps"] > 2
    assert np.all(np.isfinite(ref["state"]))
    assert rel_l2(ref["state"], c0).max() > 1e-4, "the reference solver did not move the state"
    s64, n64, t64 = ours(mesh, p, _ffi.FP64, c0, t_end)
    s32, n32, _ = ours(mesh, p, _ffi.FP32, c0, t_end)
    s32c, n32c, _ = ours(mesh, p, _ffi.FP32_COMP, c0, t_end)
    assert n64 == ref["steps"] and n32 == ref["steps"] and n32c == ref["steps"]
    assert t64 == pytest.approx(t_end, rel=1e-12)
    err64 = rel_l2(s64, ref["state"]).max()
    err32 = rel_l2(s32, ref["state"]).max()
    err32c = rel_l2(s32c, ref["state"]).max()
    print(f"{case[0]}: {ref['steps']} steps, FP64 vs reference {err64:.2e}, FP32 vs reference {err32:.2e}, "
          f"compensated FP32 vs reference {err32c:.2e}")
    assert err64 <= 1e-9, err64
    assert err32 <= 1e-5, err32
    assert err32c <= 1e-5, err32c


@pytest.mark.parametrize("case", [
    ("vortex", 16, 10.0, 2, _ffi.IC_VORTEX, VORTEX, 0.25),
    ("density wave", 12, 1.0, 3, _ffi.IC_DENSITY_WAVE, WAVE, 0.02),
], ids=lambda c: c[0])
def test_rk2_matches_reference_gpu_solver(ref_gpu, case):
    """RK2 midpoint on periodic meshes against the reference's own
    time_integrate_rk2 (src/2d/conservation/time_integrator.cu:466-614): the
    same CFL rule, steps and end time."""
    _, n, L, p, ic, params, t_end = case
    mesh = periodic_square(n, lx=L, ly=L, jitter=0.15, seed=21 + n)
    init = Solver(mesh, p, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP64)
    init.project(ic, params)
    c0 = init.get_state()
    init.close()
    ref = ref_gpu.run(mesh, p, c0, t_end, rk2=True)
    assert ref["steps"] > 2
    assert rel_l2(ref["state"], c0).max() > 1e-4, "the reference solver did not move the state"
    s64, n64, t64 = ours(mesh, p, _ffi.FP64, c0, t_end, _ffi.RK2)
    s32, n32, _ = ours(mesh, p, _ffi.FP32, c0, t_end, _ffi.RK2)
    assert n64 == ref["steps"] and n32 == ref["steps"]
    assert t64 == pytest.approx(t_end, rel=1e-12)
    err64 = rel_l2(s64, ref["state"]).max()
    err32 = rel_l2(s32, ref["state"]).max()
    print(f"rk2 {case[0]}: {ref['steps']} steps, FP64 vs reference {err64:.2e}, FP32 vs reference {err32:.2e}")
    assert err64 <= 1e-9, err64
    assert err32 <= 1e-5, err32


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_advection_matches_reference_gpu_solver(ref_gpu, p):
    n = 16
    mesh = periodic_square(n, jitter=0.15, seed=40 + p)
    init = Solver(mesh, p, _ffi.ADVECTION, _ffi.FLUX_CENTRAL, _ffi.FP64)
    init.project(_ffi.IC_GAUSSIAN, (0.4, 0.6, 0.02, 1.0, 1.0))
    c0 = init.get_state()
    init.close()
    dt = 0.1 * (1.0 / n) / (np.sqrt(2.0) * (2 * p + 1))
    steps = 25
    ref = ref_gpu.run_advection(mesh, p, c0, dt, steps)
    assert ref["steps"] == steps
    assert np.all(np.isfinite(ref["state"]))
    moved = np.linalg.norm(ref["state"] - c0.reshape(-1)) / np.linalg.norm(c0)
    assert moved > 1e-3, "the reference solver did not move the state"
    errs = {}
    for name, prec in (("fp64", _ffi.FP64), ("fp32", _ffi.FP32)):
        sv = Solver(mesh, p, _ffi.ADVECTION, _ffi.FLUX_CENTRAL, prec)
        sv.set_state(c0)
        sv.set_dt(dt)
        k, _ = sv.run(max_steps=steps)
        assert k == steps
        s_ = sv.get_state().reshape(-1)
        sv.close()
        errs[name] = np.linalg.norm(s_ - ref["state"]) / np.linalg.norm(ref["state"])
    print(f"advection p={p}: {steps} steps, FP64 vs reference {errs['fp64']:.2e}, "
          f"FP32 vs reference {errs['fp32']:.2e}")
    assert errs["fp64"] <= 1e-9, errs
    assert errs["fp32"] <= 1e-5, errs


def walled_square(n, seed):
    """[0,1]^2 in n x n cells, interior vertices jittered by 0.15 h, two
    counter-clockwise triangles per cell, numbered by the reference's
    converter's rules (from_triangles); every boundary side -1 with right
    side number 0, as in the reference's mesh files."""
    rng = np.random.default_rng(seed)
    g = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(g, g, indexing="xy")
    inner = (X > 0) & (X < 1) & (Y > 0) & (Y < 1)
    X = X + inner * rng.uniform(-0.15, 0.15, X.shape) / n
    Y = Y + inner * rng.uniform(-0.15, 0.15, Y.shape) / n
    xy = np.stack([X.ravel(), Y.ravel()], axis=1)
    v = lambda i, j: j * (n + 1) + i
    tris = []
    for j in range(n):
        for i in range(n):
            tris.append((v(i, j), v(i + 1, j), v(i + 1, j + 1)))
            tris.append((v(i, j), v(i + 1, j + 1), v(i, j + 1)))
    return from_triangles(xy, tris, lambda a, b: -1)


@pytest.mark.parametrize("p", [0, 1, 2, 3])
def test_advection_boundary_matches_reference_gpu_solver(ref_gpu, p):
    """A pulse on the reference's linear state x + y in a walled square: its
    boundary sides take the reference's exact data x - 2t + y."""
    n = 12
    mesh = walled_square(n, seed=50 + p)
    assert (mesh.right_elem < 0).sum() == 4 * n
    init = Solver(mesh, p, _ffi.ADVECTION, _ffi.FLUX_CENTRAL, _ffi.FP64)
    init.project(_ffi.IC_GAUSSIAN, (0.4, 0.6, 0.02, 0.0, 0.0))
    pulse = init.get_state()
    init.project(_ffi.IC_LINEAR, (0.0, 1.0, 1.0))
    c0 = pulse + init.get_state()
    init.close()
    dt = 0.1 * (1.0 / n) / (np.sqrt(2.0) * (2 * p + 1))
    steps = 25
    ref = ref_gpu.run_advection(mesh, p, c0, dt, steps)
    assert ref["steps"] == steps
    assert np.all(np.isfinite(ref["state"]))
    errs = {}
    for name, prec in (("fp64", _ffi.FP64), ("fp32", _ffi.FP32)):
        sv = Solver(mesh, p, _ffi.ADVECTION, _ffi.FLUX_CENTRAL, prec)
        sv.set_boundary(_ffi.BC_EXACT, _ffi.IC_LINEAR, (0.0, 1.0, 1.0))
        sv.set_option(_ffi.OPT_STAGE_TIME, _ffi.STAGE_TIME_REFERENCE)
        sv.set_state(c0)
        sv.set_dt(dt)
        k, _ = sv.run(max_steps=steps)
        assert k == steps
        s_ = sv.get_state().reshape(-1)
        sv.close()
        errs[name] = np.linalg.norm(s_ - ref["state"]) / np.linalg.norm(ref["state"])
    # the boundary data matter: with the interior trace as ghost the state differs
    sv = Solver(mesh, p, _ffi.ADVECTION, _ffi.FLUX_CENTRAL, _ffi.FP64)
    sv.set_state(c0)
    sv.set_dt(dt)
    sv.run(max_steps=steps)
    off = np.linalg.norm(sv.get_state().reshape(-1) - ref["state"]) / np.linalg.norm(ref["state"])
    sv.close()
    print(f"advection with boundary p={p}: {steps} steps, FP64 vs reference {errs['fp64']:.2e}, "
          f"FP32 vs reference {errs['fp32']:.2e} (interior-trace ghost: {off:.2e})")
    assert off > 1e3 * max(errs["fp64"], 1e-12)
    assert errs["fp64"] <= 1e-9, errs
    assert errs["fp32"] <= 1e-5, errs
