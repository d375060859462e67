"""dgx_conserved_totals (FP64 device reduction) against the oracle's totals of
the same coefficients and against the analytic totals of the density wave.

The density wave rho = 1 + 0.2 sin(2 pi (x + y)), u = v = 1, p = 1, gamma =
1.4 on the unit square has the totals  int rho = int rho u = int rho v = 1,
int E = p/(gamma-1) + rho (u^2+v^2)/2 = 2.5 + 1 = 3.5  (the sine integrates to
0 over the periodic square).  The projection with the degree-2p rule keeps
them to 1e-15 at p = 3 on a 2 x 64^2 mesh (oracle); the FP32 state rounds the
coefficients, so the FP32 path holds them to 1e-6.
"""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square, scramble
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

WAVE = (0.2, 1.0, 1.0, 1.0, 1.0)
EXACT = np.array([1.0, 1.0, 1.0, 3.5])


@pytest.mark.parametrize("precision,tol", [(_ffi.FP32, 1e-6), (_ffi.FP64, 2e-12)], ids=["fp32", "fp64"])
@pytest.mark.parametrize("n,p", [(64, 3), (37, 2), (50, 4)])
def test_totals_match_oracle_and_analytic(n, p, precision, tol, gpu, oracle_mod):
    orc = oracle_mod
    m = scramble(periodic_square(n, jitter=0.15, seed=5), seed=6)
    sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision)
    sv.project(_ffi.IC_DENSITY_WAVE, WAVE)
    got = sv.totals()
    o = orc.Oracle(m, p, orc.EULER, orc.LLF)
    # the oracle's totals of the GPU's own coefficients: the reduction alone
    np.testing.assert_allclose(got, o.totals(sv.get_state()), rtol=1e-13, atol=1e-13)
    # against the analytic totals: the projection and, for FP32, its rounding
    np.testing.assert_allclose(got, EXACT, rtol=tol, atol=0)
    # after steps: still the oracle's totals of the stepped state, and conserved
    sv.set_dt(None)
    sv.run(max_steps=5)
    got2 = sv.totals()
    np.testing.assert_allclose(got2, o.totals(sv.get_state()), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(got2, EXACT, rtol=tol, atol=0)


def test_totals_advection_gaussian(gpu, oracle_mod):
    orc = oracle_mod
    m = periodic_square(40, jitter=0.1, seed=9)
    sv = Solver(m, 2, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP64)
    sv.project(_ffi.IC_GAUSSIAN, (0.5, 0.5, 0.01, 1.0, 1.0))
    o = orc.Oracle(m, 2, orc.ADVECTION, orc.LLF)
    c0 = o.project(orc.IC_GAUSSIAN, (0.5, 0.5, 0.01, 1.0, 1.0))
    got = sv.totals()
    np.testing.assert_allclose(got, o.totals(c0), rtol=1e-13, atol=0)
    # int exp(-r^2 / 0.01) over the plane is 0.01 pi; the periodic images add
    # terms below 1e-20
    np.testing.assert_allclose(got[0], 0.01 * np.pi, rtol=1e-9)


def test_totals_allocate_once(gpu):
    """The scratch of dgx_conserved_totals is allocated on the first call and
    reused: later calls leave the device's free memory unchanged."""
    m = periodic_square(256)
    sv = Solver(m, 1, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    sv.project(_ffi.IC_DENSITY_WAVE, WAVE)
    first = sv.totals()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        np.testing.assert_array_equal(sv.totals(), first)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
