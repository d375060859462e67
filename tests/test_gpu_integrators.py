"""RK2 midpoint and forward Euler on the GPU: against the reference's own
forward-Euler output (golden vectors) and against the oracle; the stage-time
rules for time-dependent boundary data; stage-level API and the end-time
guard of the forward-Euler commit."""
import glob
import os

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.batch import Batch
from dgcuda_gb300.mesh import Mesh, dirichlet_square, periodic_square, scramble
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "euler_*.npz")))
INTEGRATORS = [(_ffi.RK2, "rk2"), (_ffi.FE, "fe")]


def rel_l2(a, b):
    nv = a.shape[0]
    a = a.reshape(nv, -1)
    b = b.reshape(nv, -1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def f32(c):
    return c.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_forward_euler_matches_reference_output(path, precision, gpu):
    z = np.load(path)
    p = int(z["p"])
    m = Mesh(*z["V"], *z["elem_s"], *z["sides"])
    sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision, 1.4, integrator=_ffi.FE)
    sv.set_state(z["c0"])
    sv.set_dt(float(z["dt"]))
    for _ in range(int(z["nsteps"])):
        sv.step()
    tol = 1e-5 if precision == _ffi.FP32 else 1e-9
    assert rel_l2(sv.get_state(), z["ref_c_fe"]).max() <= tol


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("integrator,name", INTEGRATORS, ids=[n for _, n in INTEGRATORS])
@pytest.mark.parametrize("equation,p", [(_ffi.EULER, 2), (_ffi.EULER, 3), (_ffi.ADVECTION, 4)],
                         ids=["euler-p2", "euler-p3", "advection-p4"])
def test_cfl_run_matches_oracle(equation, p, integrator, name, precision, gpu, oracle_mod):
    orc = oracle_mod
    if equation == _ffi.EULER:
        m = scramble(periodic_square(4, lx=10.0, ly=10.0, jitter=0.15, seed=p), seed=p)
        ic, params, flux, a = orc.IC_VORTEX, (5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0), orc.LLF, (1.0, 1.0)
        t_end = 0.3
    else:
        m = scramble(periodic_square(5, jitter=0.15, seed=p), seed=p)
        ic, params, flux, a = orc.IC_GAUSSIAN, (0.5, 0.5, 0.02, 1.0, 1.0), orc.LLF, (1.0, 0.5)
        t_end = 0.05
    o = orc.Oracle(m, p, equation, flux, a=a)
    o.set_integrator(integrator)
    c = o.project(ic, params)
    if precision == _ffi.FP32:
        c = f32(c)
    # forward Euler is only conditionally stable for DG: keep its runs short
    cfl = 0.7 if integrator == _ffi.RK2 else 0.1
    ref, n, t = o.run(c, t_end, cfl=cfl)
    sv = Solver(m, p, equation, flux, precision, a=a, integrator=integrator)
    sv.set_state(c)
    sv.set_dt(cfl=cfl)
    n2, t2 = sv.run(t_end=t_end)
    assert n2 == n and abs(t2 - t) <= 1e-12
    assert rel_l2(sv.get_state(), ref).max() <= (1e-5 if precision == _ffi.FP32 else 1e-11)


@pytest.mark.parametrize("integrator,name", [(_ffi.RK4, "rk4"), (_ffi.RK2, "rk2"), (_ffi.FE, "fe")],
                         ids=["rk4", "rk2", "fe"])
@pytest.mark.parametrize("rule", [_ffi.STAGE_TIME_EXACT, _ffi.STAGE_TIME_REFERENCE],
                         ids=["exact", "reference"])
def test_stage_time_rules_with_exact_dirichlet(rule, integrator, name, gpu, oracle_mod):
    orc = oracle_mod
    m = dirichlet_square(6, jitter=0.15, seed=9)
    a, params = (1.0, 0.5), (0.85, 0.5, 0.02, 0.0, 0.0)
    o = orc.Oracle(m, 3, orc.ADVECTION, orc.LLF, a=a)
    o.set_boundary(2, orc.IC_GAUSSIAN, params)
    o.set_integrator(integrator, reference_stage_time=rule == _ffi.STAGE_TIME_REFERENCE)
    c = o.project(orc.IC_GAUSSIAN, params)
    dt = 1e-3 if integrator != _ffi.FE else 2e-4
    ref, n, _ = o.run(c, 0.02, dt=dt)
    sv = Solver(m, 3, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP64, a=a, integrator=integrator)
    sv.set_boundary(_ffi.BC_EXACT, _ffi.IC_GAUSSIAN, params)
    sv.set_option(_ffi.OPT_STAGE_TIME, rule)
    sv.set_state(c)
    sv.set_dt(dt)
    n2, _ = sv.run(t_end=0.02)
    assert n2 == n
    assert rel_l2(sv.get_state(), ref).max() <= 1e-11


def test_stage_time_rule_leaves_periodic_runs_bitwise(gpu):
    m = periodic_square(8, jitter=0.1, seed=3)
    out = []
    for rule in (_ffi.STAGE_TIME_EXACT, _ffi.STAGE_TIME_REFERENCE):
        sv = Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32, integrator=_ffi.RK2)
        sv.set_option(_ffi.OPT_STAGE_TIME, rule)
        sv.project(_ffi.IC_DENSITY_WAVE, (0.2, 1.0, 0.5, 1.0, 1.0))
        sv.set_dt(cfl=0.7)
        sv.run(max_steps=20)
        out.append(sv.get_state())
    np.testing.assert_array_equal(out[0], out[1])


@pytest.mark.parametrize("integrator,nst", [(_ffi.RK4, 4), (_ffi.RK2, 2), (_ffi.FE, 1)], ids=["rk4", "rk2", "fe"])
def test_stages_compose_to_step(integrator, nst, gpu):
    m = periodic_square(6, jitter=0.1, seed=5)
    res = []
    for by_stage in (False, True):
        sv = Solver(m, 3, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32, integrator=integrator)
        sv.project(_ffi.IC_DENSITY_WAVE, (0.2, 1.0, 0.5, 1.0, 1.0))
        sv.set_dt(cfl=0.3)
        for _ in range(3):
            if by_stage:
                for s in range(nst):
                    sv.rk_stage(s)
            else:
                sv.step()
        res.append(sv.get_state())
        with pytest.raises(_ffi.DgxError):
            sv.rk_stage(nst)
    np.testing.assert_array_equal(res[0], res[1])


@pytest.mark.parametrize("integrator", [_ffi.RK2, _ffi.FE], ids=["rk2", "fe"])
def test_steps_after_end_time_leave_state(integrator, gpu):
    """At the end time dt is 0: the stages write nothing and forward Euler's
    commit is skipped, so extra steps leave the state untouched."""
    m = periodic_square(6, jitter=0.1, seed=7)
    sv = Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32, integrator=integrator)
    sv.project(_ffi.IC_DENSITY_WAVE, (0.2, 1.0, 0.5, 1.0, 1.0))
    sv.set_dt(cfl=0.2)
    n, t = sv.run(t_end=0.01)
    assert n > 0 and t == 0.01
    c = sv.get_state()
    for _ in range(3):
        sv.step()
    np.testing.assert_array_equal(sv.get_state(), c)
    assert sv.time()[0] == 0.01


def test_batch_refuses_other_integrators(gpu):
    m = periodic_square(4, seed=1)
    a = Solver(m, 1, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    b = Solver(m, 1, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32, integrator=_ffi.RK2)
    with pytest.raises(_ffi.DgxError) as ei:
        Batch([a, b])
    assert ei.value.status == _ffi.ERR_UNSUPPORTED
