"""The benchmark configurations at their stated sizes, FP32 CUDA path (through
the C ABI) against the FP64 CPU oracle run on the same inputs:

  config 2  isentropic vortex, [0,10]^2 periodic, 2 x 128^2 triangles jittered
            +-0.15h, p = 2, LLF, CFL 0.7 to t = 2 (about 1,600 steps), also
            against the exactly advected vortex;
  config 3  density wave, [0,1]^2 periodic, 2 x 1024^2 triangles jittered
            +-0.15h, p = 3, LLF, 100 RK4 steps at the first CFL dt, with the
            drift of the conserved totals.

Tolerances: relative L2 per conserved variable <= 1e-5 against the oracle;
conserved-total drift <= 1e-6 relative.  The oracle takes about half a minute
(config 2) and two to three minutes (config 3) on 16 host cores.
"""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu, pytest.mark.slow]

FP32_TOL = 1e-5
DRIFT_TOL = 1e-6
VORTEX = (5.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0)
WAVE = (0.2, 1.0, 1.0, 1.0, 1.0)


def test_config2_vortex_full_size(gpu, oracle_mod):
    orc = oracle_mod
    m = periodic_square(128, lx=10.0, ly=10.0, jitter=0.15, seed=12347)
    o = orc.Oracle(m, 2, orc.EULER, orc.LLF)
    c0 = o.project(orc.IC_VORTEX, VORTEX)
    sv = Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    sv.set_state(c0)
    sv.set_dt(None)
    n, t = sv.run(t_end=2.0)
    got = sv.get_state()
    ref, nref, tref = o.run(c0, t_end=2.0)
    assert n == nref and abs(t - 2.0) < 1e-12 and abs(tref - 2.0) < 1e-12
    err = orc.rel_l2(got, ref)
    assert err.max() <= FP32_TOL, err
    # the exact solution: the vortex advected by the free stream (1, 0) for t = 2
    exact = o.project(orc.IC_VORTEX, (7.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0))
    e_gpu, e_orc = orc.rel_l2(got, exact), orc.rel_l2(ref, exact)
    # the discretisation error of the scheme (2e-6 .. 1.5e-5 per variable), the
    # same for the FP32 path as for the FP64 oracle to within the FP32 rounding
    assert e_orc.max() <= 2e-5, e_orc
    assert np.all(np.abs(e_gpu - e_orc) <= 1e-6), (e_gpu, e_orc)


def test_config3_density_wave_100_steps_full_size(gpu, oracle_mod):
    orc = oracle_mod
    m = periodic_square(1024, jitter=0.15, seed=12347)
    o = orc.Oracle(m, 3, orc.EULER, orc.LLF)
    c0 = o.project(orc.IC_DENSITY_WAVE, WAVE).astype(np.float32).astype(np.float64)
    dt = o.cfl_dt(c0)
    sv = Solver(m, 3, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    sv.set_state(c0)
    t0 = sv.totals()
    sv.set_dt(dt)
    k, _ = sv.run(max_steps=100)
    assert k == 100
    got = sv.get_state()
    t1 = sv.totals()
    sv.close()
    ref = o.step(c0, dt)
    for _ in range(99):
        ref = o.step(ref, dt)
    err = orc.rel_l2(got, ref)
    assert err.max() <= FP32_TOL, err
    drift = np.abs(t1 - t0) / np.maximum(np.abs(t0), abs(t0[0]))
    assert drift.max() <= DRIFT_TOL, drift
    # the oracle's own totals are conserved to FP64 rounding
    tr0, tr1 = o.totals(c0), o.totals(ref)
    assert np.abs(tr1 - tr0).max() <= 1e-12 * np.abs(tr0).max()
