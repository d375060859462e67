"""The benchmark configurations at their stated sizes, FP32 CUDA path (through
the C ABI) against the FP64 CPU oracle run on the same inputs:

  config 2  isentropic vortex, [0,10]^2 periodic, 2 x 128^2 triangles jittered
            +-0.15h, p = 2, LLF, CFL 0.7 to t = 2 (about 1,600 steps), also
            against the exactly advected vortex;
  config 3  density wave, [0,1]^2 periodic, 2 x 1024^2 triangles jittered
            +-0.15h, p = 3, LLF, 100 RK4 steps at the first CFL dt, with the
            drift of the conserved totals.

Tolerances (relative L2 per conserved variable against the oracle): config 3
FP32 <= 1e-5 with conserved-total drift <= 1e-6 relative; config 2 FP64
<= 1e-9, FP32 <= 3e-4 (its ~1,630 steps accumulate the FP32 rounding of the
stored state, see the test) and compensated FP32 <= 1e-5.  The oracle takes about ten seconds (config 2) and three minutes
(config 3) on 16 host cores.
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
    """About 1,630 CFL steps.  The FP64 path matches the oracle to 1e-9.  The
    plain FP32 path's rounding accumulates over so long a run: measured on
    GB300 2.7e-5 / 4.3e-5 / 1.4e-4 / 1.8e-5 (rho, rho u, rho v, E) against the
    oracle, largest for rho v, whose free-stream value is 0.  The source is the
    FP32 rounding of the stored state that the RK4 sum accumulates, step after
    step (an FP64 run with its stored stage outputs rounded to FP32 shows the
    same error; with only the right-hand sides' inputs rounded, 1e-7), so the
    compensated FP32 precision, which keeps the increments apart from the
    state and the state as c + lo, holds this run to 1e-5.  Bounds: FP64
    <= 1e-9; FP32 <= 3e-4; compensated FP32 <= 1e-5."""
    orc = oracle_mod
    m = periodic_square(128, lx=10.0, ly=10.0, jitter=0.15, seed=12347)
    o = orc.Oracle(m, 2, orc.EULER, orc.LLF)
    c0 = o.project(orc.IC_VORTEX, VORTEX)
    ref, nref, tref = o.run(c0, t_end=2.0)
    assert abs(tref - 2.0) < 1e-12
    # the exact solution: the vortex advected by the free stream (1, 0) for t = 2
    exact = o.project(orc.IC_VORTEX, (7.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0))
    e_orc = orc.rel_l2(ref, exact)
    # the discretisation error of the scheme: 2e-6 .. 1.5e-5 per variable
    assert e_orc.max() <= 2e-5, e_orc
    names = {_ffi.FP64: "fp64", _ffi.FP32: "fp32", _ffi.FP32_COMP: "fp32 compensated"}
    for precision, tol in ((_ffi.FP64, 1e-9), (_ffi.FP32, 3e-4), (_ffi.FP32_COMP, 1e-5)):
        sv = Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, precision)
        sv.set_state(c0)
        sv.set_dt(None)
        n, t = sv.run(t_end=2.0)
        got = sv.get_state()
        sv.close()
        assert n == nref and abs(t - 2.0) < 1e-12
        err = orc.rel_l2(got, ref)
        print(f"config 2 {names[precision]}: {n} steps, rel L2 vs oracle {err}, "
              f"vs exact {orc.rel_l2(got, exact)} (oracle vs exact {e_orc})")
        assert err.max() <= tol, err


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
