"""The p = 1 slope limiter and the convergence monitor on the GPU, against the
oracle and numpy."""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.batch import Batch
from dgcuda_gb300.mesh import dirichlet_square, periodic_square, scramble
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    nv = a.shape[0]
    a = a.reshape(nv, -1)
    b = b.reshape(nv, -1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def rough_state(o, m, nv):
    rng = np.random.default_rng(7)
    c = np.zeros(o.shape)
    c[:, 0, :] = 1.0 + 0.5 * (rng.random((nv, m.num_elem)) > 0.5)
    c[:, 1:, :] = 0.4 * rng.standard_normal((nv, 2, m.num_elem))
    return c


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("equation", [_ffi.ADVECTION, _ffi.EULER], ids=["advection", "euler"])
def test_limit_matches_oracle(equation, precision, gpu, oracle_mod):
    orc = oracle_mod
    m = scramble(dirichlet_square(12, jitter=0.2, seed=1), seed=2)
    o = orc.Oracle(m, 1, equation, orc.LLF)
    c = rough_state(o, m, o.nv)
    if precision == _ffi.FP32:
        c = c.astype(np.float32).astype(np.float64)
    sv = Solver(m, 1, equation, _ffi.FLUX_LLF, precision)
    sv.set_state(c)
    sv.limit()
    ref = o.limit(c)
    got = sv.get_state()
    tol = 1e-6 if precision == _ffi.FP32 else 1e-14
    np.testing.assert_allclose(got, ref, rtol=tol, atol=tol)
    assert np.abs(ref - c).max() > 0.1


@pytest.mark.parametrize("integrator", [_ffi.RK4, _ffi.RK2], ids=["rk4", "rk2"])
def test_limited_run_matches_oracle(integrator, gpu, oracle_mod):
    orc = oracle_mod
    m = scramble(periodic_square(12, jitter=0.15, seed=3), seed=4)
    o = orc.Oracle(m, 1, orc.ADVECTION, orc.LLF, a=(1.0, 0.5))
    o.set_integrator(integrator)
    o.set_limiter(True)
    c = o.limit(rough_state(o, m, 1))
    ref, n, _ = o.run(c, 0.05, cfl=0.3)
    sv = Solver(m, 1, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP64, a=(1.0, 0.5), integrator=integrator)
    sv.set_option(_ffi.OPT_LIMITER, 1)
    sv.set_state(c)
    sv.set_dt(cfl=0.3)
    n2, _ = sv.run(t_end=0.05)
    assert n2 == n
    assert rel_l2(sv.get_state(), ref).max() <= 1e-11


def test_limiter_refusals(gpu):
    m = periodic_square(4)
    with pytest.raises(_ffi.DgxError) as ei:
        Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32).limit()
    assert ei.value.status == _ffi.ERR_UNSUPPORTED
    sv = Solver(m, 1, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    sv.set_option(_ffi.OPT_LIMITER, 1)
    with pytest.raises(_ffi.DgxError) as ei:
        Batch([sv])
    assert ei.value.status == _ffi.ERR_UNSUPPORTED


def test_state_change_matches_numpy(gpu):
    m = periodic_square(10, jitter=0.1, seed=5)
    sv = Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    sv.project(_ffi.IC_DENSITY_WAVE, (0.2, 1.0, 1.0, 1.0, 1.0))
    c0 = sv.get_state()
    prev = torch.tensor(c0, dtype=torch.float32, device="cuda")
    sv.set_dt(cfl=0.5)
    sv.run(max_steps=3)
    chg = sv.state_change(prev.data_ptr())
    ref = np.abs(sv.get_state() - c0.astype(np.float32).astype(np.float64)).max()
    assert chg == pytest.approx(ref, rel=1e-12)


def test_run_steady_stops_at_the_tolerance(gpu):
    """A pulse advected out of a box with exact inflow data leaves a steady
    (zero) state: the run stops once one step changes no coefficient by more
    than the tolerance; with tolerance 0 it runs its step limit."""
    m = dirichlet_square(12, jitter=0.1, seed=6)
    params = (0.3, 0.3, 0.005, 0.0, 0.0)

    def solver():
        sv = Solver(m, 2, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP64, a=(1.0, 1.0))
        sv.set_boundary(_ffi.BC_EXACT, _ffi.IC_GAUSSIAN, params)
        sv.project(_ffi.IC_GAUSSIAN, params)
        sv.set_dt(cfl=0.5)
        return sv

    sv = solver()
    n, chg = sv.run_steady(1e-10, 20000)
    assert chg <= 1e-10 and 10 < n < 20000
    assert np.abs(sv.get_state()).max() < 1e-6
    n, chg = solver().run_steady(0.0, 3)
    assert n == 3 and chg > 0
