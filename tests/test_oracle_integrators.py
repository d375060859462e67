"""The oracle's RK2 midpoint and forward-Euler integrators and its stage-time
rules: exact composition of RHS evaluations, temporal convergence orders, and
the reference's stage-time arguments for time-dependent boundary data."""
import numpy as np
import pytest

from dgcuda_gb300.mesh import dirichlet_square, periodic_square


def test_rk2_is_midpoint_composition(oracle_mod):
    orc = oracle_mod
    m = periodic_square(4, jitter=0.15, seed=2)
    o = orc.Oracle(m, 2, orc.EULER, orc.LLF)
    c = o.project(orc.IC_DENSITY_WAVE, (0.2, 1.0, 0.5, 1.0, 1.0))
    dt = 1e-3
    o.set_integrator(orc.RK2)
    got = o.step(c, dt)
    k1 = o.rhs(c, dt)
    want = c + o.rhs(c + 0.5 * k1, dt)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-15)
    o.set_integrator(orc.FE)
    np.testing.assert_allclose(o.step(c, dt), c + k1, rtol=0, atol=1e-15)


@pytest.mark.parametrize("integrator,order", [(2, 1), (1, 2), (0, 4)], ids=["fe", "rk2", "rk4"])
def test_temporal_order(integrator, order, oracle_mod):
    """Error against a fine RK4 solution halves by 2^order when dt halves."""
    orc = oracle_mod
    m = periodic_square(6, jitter=0.1, seed=4)
    o = orc.Oracle(m, 2, orc.ADVECTION, orc.LLF, a=(1.0, 0.5))
    c0 = o.project(orc.IC_GAUSSIAN, (0.5, 0.5, 0.05, 1.0, 1.0))
    t_end = 0.04
    ref, _, _ = o.run(c0, t_end, dt=t_end / 256)
    o.set_integrator(integrator)
    errs = []
    for n in (8, 16):
        c, steps, _ = o.run(c0, t_end, dt=t_end / n)
        assert steps == n
        errs.append(np.linalg.norm(c - ref))
    rate = np.log2(errs[0] / errs[1])
    assert abs(rate - order) < 0.3, (errs, rate)


def test_reference_stage_times(oracle_mod):
    """Stage-time rules on advection with exact, time-dependent Dirichlet data:
    exact nodes t_n + c_s dt by default; the reference's t_n for every stage."""
    orc = oracle_mod
    m = dirichlet_square(4, jitter=0.1, seed=6)
    params = (0.9, 0.5, 0.02)
    o = orc.Oracle(m, 2, orc.ADVECTION, orc.LLF, a=(1.0, 0.5))
    o.set_boundary(2, orc.IC_GAUSSIAN, params)
    c = o.project(orc.IC_GAUSSIAN, params)
    dt, t = 2e-3, 0.1
    for integrator, nodes in ((1, (0.0, 0.5)), (2, (0.0,))):
        o.set_integrator(integrator)
        got = o.step(c, dt, t=t)
        o.set_integrator(integrator, reference_stage_time=True)
        got_ref = o.step(c, dt, t=t)
        k = [o.rhs(c, dt, t + nodes[0] * dt)]
        kr = [o.rhs(c, dt, t)]
        if integrator == 1:
            want = c + o.rhs(c + 0.5 * k[0], dt, t + 0.5 * dt)
            want_ref = c + o.rhs(c + 0.5 * kr[0], dt, t)
        else:
            want, want_ref = c + k[0], c + kr[0]
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-15)
        np.testing.assert_allclose(got_ref, want_ref, rtol=0, atol=1e-15)
        if integrator == 1:   # the second stage's boundary data moves in time
            assert np.abs(got - got_ref).max() > 0


def test_reference_stage_times_euler(oracle_mod):
    """Euler RK4 under the reference rule evaluates stage s at t_{n+1} + c_s dt."""
    orc = oracle_mod
    m = periodic_square(3, jitter=0.1, seed=8)
    o = orc.Oracle(m, 1, orc.EULER, orc.LLF)
    c = o.project(orc.IC_DENSITY_WAVE, (0.2, 1.0, 0.5, 1.0, 1.0))
    o.set_integrator(orc.RK4, reference_stage_time=True)
    # periodic: no boundary data, so the rule changes nothing
    a = o.step(c, 1e-3, t=0.3)
    o.set_integrator(orc.RK4)
    np.testing.assert_array_equal(a, o.step(c, 1e-3, t=0.3))
