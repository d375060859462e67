"""The reference's problem plug-ins on the GPU against the oracle: cylinder
(RK2, as cylinder.cu runs it), supersonic vortex and three-point shock, each
with its own initial state and ghost states (DGX_BC_PROBLEM)."""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import annulus, dirichlet_square, scramble, tag_boundary
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SUPERSONIC = (2.25, 1.0125)
THREEPOINT = (0.25, 5.0)
CYLINDER = (0.38,)


def rel_l2(a, b):
    nv = a.shape[0]
    a = a.reshape(nv, -1)
    b = b.reshape(nv, -1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def gpu_rhs(sv, c, t=0.0):
    dtype = torch.float64 if sv.precision == _ffi.FP64 else torch.float32
    u = torch.tensor(np.ascontiguousarray(c), dtype=dtype, device="cuda")
    k = torch.zeros_like(u)
    sv.rhs_eval(u.data_ptr(), k.data_ptr(), 1.0, t, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return k.double().cpu().numpy()


def problem(name):
    if name == "cylinder":
        m = annulus(4, 24, 0.15, 0.5, cx=0.5, cy=0.5,
                    tag=lambda x, y, w: -1 if w == "inner" else (-3 if x < 0.5 else -2))
        return m, _ffi.IC_CYLINDER, CYLINDER, _ffi.RK2, 0.05
    if name == "supersonic":
        return annulus(4, 8, 1.0, 1.384, 0.0, np.pi / 2), _ffi.IC_SUPERSONIC_VORTEX, SUPERSONIC, _ffi.RK4, 0.02
    m = tag_boundary(dirichlet_square(6, jitter=0.1, seed=4),
                     lambda x, y: -1 if y < 1e-9 else (-3 if x < 1e-9 else -2))
    return m, _ffi.IC_THREEPOINT, THREEPOINT, _ffi.RK4, 0.2


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("name", ["cylinder", "supersonic", "threepoint"])
def test_problem_matches_oracle(name, p, precision, gpu, oracle_mod):
    orc = oracle_mod
    m, ic, params, integrator, t_end = problem(name)
    m = scramble(m, seed=p, permute=False)
    o = orc.Oracle(m, p, orc.EULER, orc.LLF)
    o.set_boundary(3, ic, params)
    o.set_integrator(integrator)
    sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision, integrator=integrator)
    sv.set_boundary(_ffi.BC_PROBLEM, ic, params)
    c = o.project(ic, params)
    sv.project(ic, params)
    # projection on the device in FP64, stored in the solver's precision
    assert rel_l2(sv.get_state(), c).max() <= (1e-7 if precision == _ffi.FP32 else 1e-13)
    # tilt the state (the supersonic vortex is an exact steady state, whose
    # RHS is rounding noise only)
    c[:, 1, :] += 0.02 * c[:, 0, :]
    if precision == _ffi.FP32:
        c = c.astype(np.float32).astype(np.float64)
    err = rel_l2(gpu_rhs(sv, c, t=0.05), o.rhs(c, 1.0, t=0.05))
    # the three-point state has an exact jump inside elements: relative errors
    # of its small RHS are larger in FP32
    tol = (5e-4 if name == "threepoint" else 1e-4) if precision == _ffi.FP32 else 1e-11
    assert err.max() <= tol, err
    ref, n, _ = o.run(c, t_end, cfl=0.5)
    sv.set_state(c)
    sv.set_dt(cfl=0.5)
    n2, _ = sv.run(t_end=t_end)
    assert n2 == n
    assert rel_l2(sv.get_state(), ref).max() <= (2e-5 if precision == _ffi.FP32 else 1e-10)


def test_problem_boundary_needs_euler_and_a_problem(gpu):
    m = annulus(2, 8, 1.0, 1.384, 0.0, np.pi / 2)
    sv = Solver(m, 1, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP32)
    with pytest.raises(_ffi.DgxError):
        sv.set_boundary(_ffi.BC_PROBLEM, _ffi.IC_SUPERSONIC_VORTEX, SUPERSONIC)
    sv = Solver(m, 1, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    with pytest.raises(_ffi.DgxError):
        sv.set_boundary(_ffi.BC_PROBLEM, _ffi.IC_VORTEX, (5, 5, 1, 1, 0, 0, 0))
