"""DGX_FP32_COMP: FP32 state and arithmetic with compensated RK4 accumulation
(the increments kept apart from the state, the state carried as c + lo and
updated by an error-free two-sum).  Through the C ABI:

  * long runs: the 2 x 128^2, p = 2 vortex to t = 2 (1,634 CFL steps) and a
    2,000-step order-3 vortex against the FP64 path, where the plain FP32
    path's stored-state rounding accumulates ~1e-5 .. 1e-4;
  * the state's two parts hold an FP64 state to ~1e-15 (set, then get);
  * batches (per-class and fused launches) and the request server give each
    compensated solve the same bits as running it alone.

Bounds are relative L2 per conserved variable: 1e-5 (the FP32 path's target)
on runs of thousands of steps, and at most a tenth of the plain FP32 path's
error; the measured values on GB300 are in each test's docstring."""
import time

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.batch import Batch
from dgcuda_gb300.mesh import periodic_square
from dgcuda_gb300.serve import Server, request
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

COMP_LONG_TOL = 1e-5


def rel_l2(a, b):
    return np.array([np.linalg.norm(a[n] - b[n]) / np.linalg.norm(b[n]) for n in range(a.shape[0])])


def long_run(m, p, params, precision, t_end=0.0, steps=0, c0=None):
    sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision)
    sv.set_state(c0)
    sv.set_dt(None)
    n, t = sv.run(t_end=t_end, max_steps=steps)
    out = sv.get_state()
    sv.close()
    return out, n, t


def initial(m, p, params):
    ref = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP64)
    ref.project(_ffi.IC_VORTEX, params)
    c0 = ref.get_state().astype(np.float32).astype(np.float64)   # exactly representable in every precision
    ref.close()
    return c0


def test_config2_long_run_against_fp64(gpu):
    """Config 2 at its stated size (1,634 steps to t = 2).  Measured on GB300
    against the FP64 path: compensated 4.5e-7 / 7.8e-7 / 1.4e-6 / 2.8e-7
    (rho, rho u, rho v, E), plain FP32 1.9e-5 / 2.6e-5 / 8.3e-5 / 1.1e-5."""
    m = periodic_square(128, lx=10.0, ly=10.0, jitter=0.15, seed=12347)
    params = (5.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0)
    c0 = initial(m, 2, params)
    ref, nref, _ = long_run(m, 2, params, _ffi.FP64, t_end=2.0, c0=c0)
    got, n, t = long_run(m, 2, params, _ffi.FP32_COMP, t_end=2.0, c0=c0)
    plain, _, _ = long_run(m, 2, params, _ffi.FP32, t_end=2.0, c0=c0)
    assert n == nref and abs(t - 2.0) < 1e-12
    err, err_plain = rel_l2(got, ref), rel_l2(plain, ref)
    print(f"config 2: compensated {err}, plain FP32 {err_plain}")
    assert err.max() <= COMP_LONG_TOL, err
    assert (err < 0.1 * err_plain).all(), (err, err_plain)


def test_2000_steps_order3_against_fp64(gpu):
    """2,000 steps of an order-3 vortex on 2 x 81^2 elements (the length of
    the served configuration's long requests), at the first step's CFL dt.
    Measured on GB300: compensated 7.4e-7 / 1.3e-6 / 4.2e-6 / 5.4e-7, plain
    FP32 2.2e-5 / 2.9e-5 / 1.5e-4 / 8.0e-6."""
    m = periodic_square(81, lx=10.0, ly=10.0, jitter=0.15, seed=778)
    params = (4.0, 5.5, 2.5, 1.0, 0.0, 10.0, 10.0)
    c0 = initial(m, 3, params)
    # a fixed dt, so both runs end at the same time
    sv = Solver(m, 3, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP64)
    sv.set_state(c0)
    sv.set_dt(None)
    sv.run(max_steps=1)
    dt = sv.time()[1]
    sv.close()
    out = {}
    for prec in (_ffi.FP64, _ffi.FP32_COMP, _ffi.FP32):
        sv = Solver(m, 3, _ffi.EULER, _ffi.FLUX_LLF, prec)
        sv.set_state(c0)
        sv.set_dt(dt)
        sv.run(max_steps=2000)
        out[prec] = sv.get_state()
        sv.close()
    err = rel_l2(out[_ffi.FP32_COMP], out[_ffi.FP64])
    err_plain = rel_l2(out[_ffi.FP32], out[_ffi.FP64])
    print(f"2000 steps: compensated {err}, plain FP32 {err_plain}")
    assert err.max() <= COMP_LONG_TOL, err
    assert (err < 0.1 * err_plain).all(), (err, err_plain)


def test_state_pair_holds_fp64_values(gpu):
    m = periodic_square(7, lx=10.0, ly=10.0, jitter=0.15, seed=3)
    sv = Solver(m, 3, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32_COMP)
    rng = np.random.default_rng(5)
    c = rng.standard_normal(sv.get_state().shape) * 3.0 + 1.0
    sv.set_state(c)
    back = sv.get_state()
    assert np.abs(back - c).max() <= 1e-13 * np.abs(c).max()
    # an FP32 upload clears the low part: the state is exactly the FP32 values
    c32 = c.astype(np.float32)
    sv.set_state_f32(np.ascontiguousarray(c32).ravel())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(sv.get_state(), c32.astype(np.float64))
    sv.close()


def test_totals_of_the_state_pair(gpu, oracle_mod):
    """dgx_conserved_totals of a compensated solver is the total of c + lo:
    equal to the oracle's totals of the FP64 state set into it."""
    m = periodic_square(9, lx=10.0, ly=10.0, jitter=0.15, seed=8)
    sv = Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32_COMP)
    o = oracle_mod.Oracle(m, 2, oracle_mod.EULER, oracle_mod.LLF)
    c = o.project(oracle_mod.IC_VORTEX, (5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0))
    sv.set_state(c)
    ref = o.totals(c)
    np.testing.assert_allclose(sv.totals(), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    sv.close()


def test_compensated_refuses_other_integrators(gpu):
    m = periodic_square(4)
    with pytest.raises(_ffi.DgxError):
        Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32_COMP, integrator=_ffi.RK2)


def _mk(case, seed, precision):
    eq, p, n = case
    if eq == _ffi.EULER:
        m = periodic_square(n, lx=10.0, ly=10.0, jitter=0.15, seed=seed)
        ic, params = _ffi.IC_VORTEX, (5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0)
    else:
        m = periodic_square(n, jitter=0.15, seed=seed)
        ic, params = _ffi.IC_GAUSSIAN, (0.3, 0.6, 0.02, 1.0, 1.0)
    sv = Solver(m, p, eq, _ffi.FLUX_LLF, precision, a=(1.0, 0.7))
    sv.project(ic, params)
    sv.set_dt(None if eq == _ffi.EULER else 1e-3)
    return sv


BATCH = [(_ffi.EULER, 3, 10), (_ffi.EULER, 2, 5), (_ffi.ADVECTION, 2, 7), (_ffi.EULER, 4, 6)]


@pytest.mark.parametrize("fused", [0, 2])
def test_batch_equals_alone(fused, gpu):
    """Compensated solves (with plain FP32 ones in the same batch) advanced by
    the batched step equal the same solves run alone, bit for bit."""
    cases = [(c, prec) for c in BATCH for prec in (_ffi.FP32_COMP, _ffi.FP32)]
    alone = [_mk(c, i, prec) for i, (c, prec) in enumerate(cases)]
    mixed = [_mk(c, i, prec) for i, (c, prec) in enumerate(cases)]
    for sv in alone:
        sv.run(max_steps=7)
    b = Batch(mixed)
    if fused:
        b.set_fused(fused)
    b.run(7)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m.get_state(), a.get_state())
    b.close()


def test_server_request_equals_alone(gpu):
    srv = Server(budget_bytes=1 << 30, max_active=16)
    srv.set_steps_per_check(3)
    sp = dict(n=9, order=3, equation=_ffi.EULER, ic=_ffi.IC_VORTEX, params=(5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0),
              t_end=0.2, lx=10.0, ly=10.0, jitter=0.15, seed=31, a=(1.0, 0.6))
    ids = [srv.submit(request(keep_state=True, precision=prec, **sp)) for prec in (_ffi.FP32_COMP, _ffi.FP32)]
    assert srv.wait_idle(60.0) == _ffi.OK
    for rid, prec in zip(ids, (_ffi.FP32_COMP, _ffi.FP32)):
        m = periodic_square(sp["n"], lx=sp["lx"], ly=sp["ly"], jitter=sp["jitter"], seed=sp["seed"])
        sv = Solver(m, sp["order"], sp["equation"], _ffi.FLUX_LLF, prec, a=sp["a"])
        sv.project(sp["ic"], sp["params"])
        sv.set_dt(None, cfl=0.7)
        n, t = sv.run(t_end=sp["t_end"])
        ref = sv.get_state()
        state, tot, steps, tfin = srv.result(rid, ref.size)
        assert steps == n and tfin == t
        np.testing.assert_array_equal(state.reshape(ref.shape), ref)
        sv.close()
    srv.close()


@pytest.mark.parametrize("kind", ["channel", "advection"])
def test_compensated_parity_with_boundaries_and_advection(kind, gpu, oracle_mod):
    """The compensated stages on a mesh with boundary sides (the kernels with
    ghost-state code: a channel with reflecting walls, free-stream inflow and
    outflow) and on advection: 10 RK4 steps against the FP64 oracle from the
    same FP64 state, within the FP32 path's bound."""
    from dgcuda_gb300.mesh import dirichlet_square, scramble, tag_boundary
    orc = oracle_mod
    o_bc = None
    if kind == "channel":
        m = dirichlet_square(6, lx=10.0, ly=10.0, jitter=0.15, seed=3)
        m = tag_boundary(m, lambda x, y: -3 if x < 1e-9 else (-2 if x > 10 - 1e-9 else -1))
        m = scramble(m, seed=3, permute=False)
        eq, ic, params = _ffi.EULER, _ffi.IC_VORTEX, (5.0, 5.0, 3.0, 0.5, 0.0, 0.0, 0.0)
        o_bc = (1.0, 0.5, 0.0, 1.0)
    else:
        m = scramble(periodic_square(9, jitter=0.15, seed=4), seed=6)
        eq, ic, params = _ffi.ADVECTION, _ffi.IC_GAUSSIAN, (0.4, 0.6, 0.05, 1.0, 1.0)
    o = orc.Oracle(m, 3, eq, orc.LLF)
    if o_bc:
        o.set_boundary(1, 0, o_bc)
    c0 = o.project(ic, params)
    dt = 0.3 * o.cfl_dt(c0) if eq == _ffi.EULER else 0.002
    ref = c0.copy()
    for s in range(10):
        ref = o.step(ref, dt, t=s * dt)
    sv = Solver(m, 3, eq, _ffi.FLUX_LLF, _ffi.FP32_COMP)
    if o_bc:
        sv.set_boundary(_ffi.BC_FREESTREAM, 0, o_bc)
    sv.set_state(c0)
    sv.set_dt(dt)
    sv.run(max_steps=10)
    err = rel_l2(sv.get_state(), ref)
    assert err.max() <= 1e-5, err
