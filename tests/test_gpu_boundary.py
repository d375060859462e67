"""Boundary sides on the GPU against the oracle: Euler reflecting walls with
free-stream inflow/outflow, advection with exact (translated) Dirichlet data,
and the steady polynomial known-answer test."""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import dirichlet_square, scramble, tag_boundary
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


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


def euler_channel(n=6, seed=3):
    m = dirichlet_square(n, lx=10.0, ly=10.0, jitter=0.15, seed=seed)
    return tag_boundary(m, lambda x, y: -3 if x < 1e-9 else (-2 if x > 10 - 1e-9 else -1))


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_euler_boundaries_match_oracle(p, precision, gpu, oracle_mod):
    orc = oracle_mod
    m = scramble(euler_channel(seed=p), seed=p, permute=False)
    fs = (1.0, 0.5, 0.0, 1.0)
    o = orc.Oracle(m, p, orc.EULER, orc.LLF)
    o.set_boundary(1, 0, fs)
    c = o.project(orc.IC_VORTEX, (5.0, 5.0, 3.0, 0.5, 0.0, 0.0, 0.0))
    if precision == _ffi.FP32:
        c = c.astype(np.float32).astype(np.float64)
    sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision)
    sv.set_boundary(_ffi.BC_FREESTREAM, 0, fs)
    err = rel_l2(gpu_rhs(sv, c), o.rhs(c)).max()
    # FP32: the vortex's volume and surface terms cancel to a small net RHS on
    # this coarse mesh, so one RHS carries up to ~1e-4 relative rounding at p = 4
    assert err <= (1e-4 if precision == _ffi.FP32 else 1e-12), err
    dt = 0.3 * o.cfl_dt(c)
    ref = c.copy()
    for s in range(10):
        ref = o.step(ref, dt, t=s * dt)
    sv.set_state(c)
    sv.set_dt(dt)
    sv.run(max_steps=10)
    assert rel_l2(sv.get_state(), ref).max() <= (1e-5 if precision == _ffi.FP32 else 1e-11)


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
def test_advection_exact_dirichlet_matches_oracle(precision, gpu, oracle_mod):
    orc = oracle_mod
    m = dirichlet_square(8, jitter=0.15, seed=5)
    a = (1.0, 0.5)
    params = (0.85, 0.5, 0.02, 0.0, 0.0)           # a pulse leaving through the right side
    o = orc.Oracle(m, 3, orc.ADVECTION, orc.LLF, a=a)
    o.set_boundary(2, orc.IC_GAUSSIAN, params)
    c = o.project(orc.IC_GAUSSIAN, params)
    if precision == _ffi.FP32:
        c = c.astype(np.float32).astype(np.float64)
    sv = Solver(m, 3, _ffi.ADVECTION, _ffi.FLUX_LLF, precision, a=a)
    sv.set_boundary(_ffi.BC_EXACT, _ffi.IC_GAUSSIAN, params)
    err = rel_l2(gpu_rhs(sv, c, t=0.1), o.rhs(c, 1.0, t=0.1)).max()
    assert err <= (5e-5 if precision == _ffi.FP32 else 1e-12), err
    dt = 2e-3
    ref, n, _ = o.run(c, t_end=0.2, dt=dt)
    sv.set_state(c)
    sv.set_dt(dt)
    n2, _ = sv.run(t_end=0.2)
    assert n2 == n
    assert rel_l2(sv.get_state(), ref).max() <= (1e-5 if precision == _ffi.FP32 else 1e-11)


@pytest.mark.parametrize("p,alpha", [(2, 2), (3, 3), (4, 4)])
def test_polynomial_steady_state_gpu(p, alpha, gpu):
    """The reference's steady advection KAT: (x - y)^alpha with a = (1,1) and
    exact Dirichlet data is unchanged by the FP64 path to rounding."""
    m = dirichlet_square(6, jitter=0.15, seed=alpha)
    sv = Solver(m, p, _ffi.ADVECTION, _ffi.FLUX_CENTRAL, _ffi.FP64, a=(1.0, 1.0))
    sv.set_boundary(_ffi.BC_EXACT, _ffi.IC_POLY, (float(alpha),))
    sv.project(_ffi.IC_POLY, (float(alpha),))
    c0 = sv.get_state()
    sv.set_dt(1e-3)
    sv.run(max_steps=50)
    np.testing.assert_allclose(sv.get_state(), c0, atol=1e-10)
