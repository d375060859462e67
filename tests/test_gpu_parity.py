"""Parity of the CUDA path (through the C ABI) with the FP64 oracle and with the
reference's own outputs (golden vectors).

Tolerances (relative L2 per conserved variable):
  states (after RK4 steps / runs), FP32 path vs FP64 oracle     <= 1e-5
    (the compensated FP32 precision too: over 10-20 steps it gains little)
  states, FP64 path vs FP64 oracle                              <= 1e-11
  one RHS, FP64 path vs FP64 oracle                             <= 1e-12
  one RHS, FP32 path vs FP64 oracle on the same FP32 input      <= 5e-5
The RHS bound is looser than the state bound because the volume and surface
terms of an element nearly cancel for smooth solutions (by a factor that grows
like 1/h), so FP32 rounding of the terms shows up relative to the small net RHS;
a step adds dt*k to a state that is much larger than dt*k, so the same rounding
stays far below 1e-5 in the states.
"""
import glob
import math
import os

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import Mesh, periodic_square, scramble
from dgcuda_gb300.solver import DeviceMesh, Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "euler_*.npz")))
FP32_TOL = 1e-5
FP32_RHS_TOL = 5e-5
FP64_TOL = 1e-12

VORTEX = (5.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0)
WAVE = (0.2, 1.0, 1.0, 1.0, 1.0)


def rel_l2(a, b):
    nv = a.shape[0]
    a = a.reshape(nv, -1)
    b = b.reshape(nv, -1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def round_state(c, precision):
    # FP32: the FP32 values; the compensated precision holds the FP64 values as c + lo
    return c.astype(np.float32).astype(np.float64) if precision == _ffi.FP32 else c


# state bounds after RK4 steps per precision (the compensated precision takes
# the FP32 bound: over 10-20 steps its gain is small)
STATE_TOL = {_ffi.FP32: FP32_TOL, _ffi.FP32_COMP: FP32_TOL, _ffi.FP64: 1e-11}


def gpu_rhs(sv, c, dt=1.0, t=0.0):
    dtype = torch.float64 if sv.precision == _ffi.FP64 else torch.float32
    u = torch.tensor(np.ascontiguousarray(c), dtype=dtype, device="cuda")
    k = torch.zeros_like(u)
    sv.rhs_eval(u.data_ptr(), k.data_ptr(), dt, t, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return k.double().cpu().numpy()


def make_case(kind, p, n=4, seed=0):
    if kind == "vortex":
        m = periodic_square(n, lx=10.0, ly=10.0, jitter=0.15, seed=seed)
        return m, _ffi.EULER, _ffi.IC_VORTEX, VORTEX
    if kind == "wave":
        m = periodic_square(n, jitter=0.15, seed=seed)
        return m, _ffi.EULER, _ffi.IC_DENSITY_WAVE, WAVE
    m = periodic_square(n, jitter=0.15, seed=seed)
    return m, _ffi.ADVECTION, _ffi.IC_GAUSSIAN, (0.4, 0.6, 0.05, 1.0, 1.0)


def test_geometry_matches_oracle(gpu, oracle_mod):
    m = scramble(periodic_square(6, jitter=0.2, seed=4), seed=2)
    g = DeviceMesh(m).geometry()
    o = oracle_mod.Oracle(m, 1, oracle_mod.EULER).geometry()
    for k in ("J", "xr", "yr", "xs", "ys", "diam", "len", "nx", "ny"):
        np.testing.assert_allclose(g[k], o[k], rtol=1e-14, atol=1e-15, err_msg=k)


@pytest.mark.parametrize("kind", ["vortex", "wave", "advection"])
def test_projection_matches_oracle(kind, gpu, oracle_mod):
    m, eq, ic, params = make_case(kind, 3, n=5, seed=1)
    sv = Solver(m, 3, eq, _ffi.FLUX_LLF, _ffi.FP64)
    sv.project(ic, params)
    o = oracle_mod.Oracle(m, 3, eq)
    np.testing.assert_allclose(sv.get_state(), o.project(ic, params), rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("flux", [_ffi.FLUX_LLF, _ffi.FLUX_CENTRAL], ids=["llf", "central"])
@pytest.mark.parametrize("kind", ["vortex", "wave", "advection"])
@pytest.mark.parametrize("p", range(6))
def test_rhs_parity(p, kind, flux, precision, gpu, oracle_mod):
    orc = oracle_mod
    m, eq, ic, params = make_case(kind, p, n=4, seed=p)
    m = scramble(m, seed=p + 10)
    a = (1.0, 0.5)
    o = orc.Oracle(m, p, eq, flux, 1.4, a=a)
    c = round_state(o.project(ic, params), precision)
    ref = o.rhs(c, 1.0)
    sv = Solver(m, p, eq, flux, precision, 1.4, a=a)
    got = gpu_rhs(sv, c)
    err = rel_l2(got, ref).max()
    assert err <= (FP32_RHS_TOL if precision == _ffi.FP32 else FP64_TOL), err


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_matches_reference_output(path, precision, gpu):
    """One RHS and a few RK4 steps against the reference's own CPU Euler code."""
    z = np.load(path)
    p = int(z["p"])
    m = Mesh(*z["V"], *z["elem_s"], *z["sides"])
    sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, precision, 1.4)
    c0 = round_state(z["c0"], precision)
    k = gpu_rhs(sv, c0)
    # the reference evaluated the unrounded FP64 state; the FP32 path sees it
    # rounded to FP32, and the RHS amplifies that input rounding
    tol = 2e-4 if precision == _ffi.FP32 else (1e-7 if p < 5 else 5e-6)
    assert rel_l2(k, z["ref_rhs"]).max() <= tol
    sv.set_state(z["c0"])
    sv.set_dt(float(z["dt"]))
    sv.set_end_time(0.0)
    for _ in range(int(z["nsteps"])):
        sv.step()
    c = sv.get_state()
    assert rel_l2(c, z["ref_c_final"]).max() <= (FP32_TOL if precision == _ffi.FP32 else 1e-9)


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64, _ffi.FP32_COMP], ids=["fp32", "fp64", "fp32comp"])
@pytest.mark.parametrize("kind,p", [("vortex", 3), ("wave", 2), ("advection", 4), ("vortex", 1)])
def test_rk4_steps_parity(kind, p, precision, gpu, oracle_mod):
    orc = oracle_mod
    m, eq, ic, params = make_case(kind, p, n=6, seed=3)
    m = scramble(m, seed=5)
    o = orc.Oracle(m, p, eq, _ffi.FLUX_LLF)
    c0 = round_state(o.project(ic, params), precision)
    dt = 0.3 * o.cfl_dt(c0) if eq == _ffi.EULER else 0.002
    ref = c0.copy()
    for s in range(20):
        ref = o.step(ref, dt)
    sv = Solver(m, p, eq, _ffi.FLUX_LLF, precision)
    sv.set_state(c0)
    sv.set_dt(dt)
    n, t = sv.run(max_steps=20)
    assert n == 20 and abs(t - 20 * dt) < 1e-12
    err = rel_l2(sv.get_state(), ref).max()
    assert err <= STATE_TOL[precision], err


def test_cfl_run_to_end_time(gpu, oracle_mod):
    """CFL-controlled run with the last step clipped to t_end: same step count,
    final time and state as the oracle (FP64 path)."""
    orc = oracle_mod
    m, eq, ic, params = make_case("vortex", 2, n=6, seed=7)
    o = orc.Oracle(m, 2, eq, orc.LLF)
    c0 = o.project(ic, params)
    t_end = 0.25
    ref, nref, tref = o.run(c0, t_end=t_end)
    sv = Solver(m, 2, eq, _ffi.FLUX_LLF, _ffi.FP64)
    sv.set_state(c0)
    sv.set_dt(None, cfl=0.7)
    n, t = sv.run(t_end=t_end)
    assert n == nref and t == tref
    assert rel_l2(sv.get_state(), ref).max() <= 1e-11
    # FP32 path on the same run
    s32 = Solver(m, 2, eq, _ffi.FLUX_LLF, _ffi.FP32)
    s32.set_state(c0)
    s32.set_dt(None, cfl=0.7)
    n32, t32 = s32.run(t_end=t_end)
    assert n32 == nref and abs(t32 - t_end) < 1e-15
    assert rel_l2(s32.get_state(), ref).max() <= FP32_TOL


def test_rk_stage_calls_equal_step(gpu):
    m, eq, ic, params = make_case("wave", 3, n=5, seed=2)
    a = Solver(m, 3, eq, _ffi.FLUX_LLF, _ffi.FP32)
    b = Solver(m, 3, eq, _ffi.FLUX_LLF, _ffi.FP32)
    for s in (a, b):
        s.project(ic, params)
        s.set_dt(1e-3)
    a.step()
    for st in range(4):
        b.rk_stage(st)
    np.testing.assert_array_equal(a.get_state(), b.get_state())


def test_deterministic_and_conservative(gpu):
    m, eq, ic, params = make_case("vortex", 3, n=16, seed=9)
    states, totals = [], []
    for _ in range(2):
        sv = Solver(m, 3, eq, _ffi.FLUX_LLF, _ffi.FP32)
        sv.project(ic, params)
        t0 = sv.totals()
        sv.set_dt(None, cfl=0.7)
        sv.run(max_steps=50)
        states.append(sv.get_state())
        totals.append((t0, sv.totals()))
    np.testing.assert_array_equal(states[0], states[1])
    t0, t1 = totals[0]
    drift = np.abs(t1 - t0) / np.maximum(np.abs(t0), 1e-300)
    # momentum-y total is ~0 for this flow; compare against the density scale
    drift[2] = abs(t1[2] - t0[2]) / abs(t0[0])
    assert drift.max() <= 1e-6, drift


def test_nonfinite_state_is_reported(gpu):
    m, eq, ic, params = make_case("wave", 2, n=4, seed=1)
    sv = Solver(m, 2, eq, _ffi.FLUX_LLF, _ffi.FP32)
    sv.project(ic, params)
    c = sv.get_state()
    c[0, 0, 5] = -1.0          # negative density injected in the host buffer
    sv.set_state(c)
    sv.set_dt(None)
    with pytest.raises(_ffi.DgxError) as ei:
        sv.run(max_steps=4)
    assert ei.value.status == _ffi.ERR_NONFINITE


def test_unsupported_requests_fail_loudly(gpu):
    m = periodic_square(3)
    with pytest.raises(_ffi.DgxError) as ei:
        Solver(m, 6, _ffi.EULER)
    assert ei.value.status == _ffi.ERR_UNSUPPORTED


def test_config1_advection(gpu, oracle_mod):
    """Config 1: advection a=(1,1), 2x32^2 periodic, p=1, LLF, dt = 0.1 h/(|a|(2p+1)),
    one period (t=1) -- FP32 GPU against the FP64 oracle and the exact solution."""
    orc = oracle_mod
    m = periodic_square(32)
    params = (0.5, 0.5, 0.01, 1.0, 1.0)
    h = 1.0 / 32
    dt = 0.1 * h / (math.sqrt(2.0) * 3)
    o = orc.Oracle(m, 1, orc.ADVECTION, orc.LLF, a=(1.0, 1.0))
    c0 = o.project(orc.IC_GAUSSIAN, params)
    ref, nref, tref = o.run(c0, t_end=1.0, dt=dt)
    sv = Solver(m, 1, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP32, a=(1.0, 1.0))
    sv.project(_ffi.IC_GAUSSIAN, params)
    sv.set_dt(dt)
    n, t = sv.run(t_end=1.0)
    assert n == nref == 1358 and abs(t - 1.0) < 1e-12
    c = sv.get_state()
    assert rel_l2(c, ref).max() <= FP32_TOL
    # after one period the exact solution is the initial condition: the
    # scheme's own error there (p = 1 on a pulse about two elements wide) is
    # 5.6 % in the coefficients' L2 norm; the GPU's equals the FP64 oracle's
    # within the parity bound (|err - err_ref| <= ||c - ref|| / ||c0||)
    err, err_ref = rel_l2(c, c0).max(), rel_l2(ref, c0).max()
    assert 0.05 < err_ref < 0.06
    assert abs(err - err_ref) <= FP32_TOL


def test_config2_vortex_reduced(gpu, oracle_mod):
    """Config 2 at a quarter of the resolution (2x32^2, p=2, t=0.5): FP32 GPU vs FP64 oracle."""
    orc = oracle_mod
    m = periodic_square(32, lx=10.0, ly=10.0, jitter=0.15, seed=12347)
    o = orc.Oracle(m, 2, orc.EULER, orc.LLF)
    c0 = o.project(orc.IC_VORTEX, VORTEX)
    ref, nref, _ = o.run(c0, t_end=0.5)
    sv = Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, _ffi.FP32)
    sv.set_state(c0)
    sv.set_dt(None)
    n, t = sv.run(t_end=0.5)
    assert n == nref and abs(t - 0.5) < 1e-12
    assert rel_l2(sv.get_state(), ref).max() <= FP32_TOL


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64, _ffi.FP32_COMP], ids=["fp32", "fp64", "fp32comp"])
@pytest.mark.parametrize("kind,p,n", [("vortex", 3, 13), ("wave", 3, 12), ("vortex", 4, 11), ("advection", 3, 13)])
def test_rk4_steps_parity_scrambled_tiles(kind, p, n, precision, gpu, oracle_mod):
    """Several tiles of a scrambled mesh (E = 2 n^2 = 242..338: up to three
    tiles whose halos hold most of their neighbours, so the trace slots past
    the tile's own 3*128 are in use), E both a multiple of 4 and not: 10 RK4
    steps against the oracle."""
    orc = oracle_mod
    m, eq, ic, params = make_case(kind, p, n=n, seed=7)
    m = scramble(m, seed=11)
    o = orc.Oracle(m, p, eq, _ffi.FLUX_LLF)
    c0 = round_state(o.project(ic, params), precision)
    dt = 0.3 * o.cfl_dt(c0) if eq == _ffi.EULER else 0.002
    ref = c0.copy()
    for s in range(10):
        ref = o.step(ref, dt)
    sv = Solver(m, p, eq, _ffi.FLUX_LLF, precision)
    sv.set_state(c0)
    sv.set_dt(dt)
    k, _ = sv.run(max_steps=10)
    assert k == 10
    err = rel_l2(sv.get_state(), ref).max()
    assert err <= STATE_TOL[precision], err


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64, _ffi.FP32_BF16X3, _ffi.FP32_COMP],
                         ids=["fp32", "fp64", "bf16x3", "fp32comp"])
@pytest.mark.parametrize("n", [8, 5, 9, 13])
def test_prefetch_option_is_bitwise_neutral(n, precision, gpu):
    """RK stages with the epilogue operands staged by the TMA engine give the
    same bits as plain loads, whatever E (= 2 n^2: 128, 50, 162, 338) is
    modulo the 16-byte alignment of the planes (the staged slices are widened
    to 16-byte boundaries and read at their offset)."""
    m, eq, ic, params = make_case("vortex", 3, n=n, seed=4)
    out = []
    for pre in (1, 0):
        sv = Solver(m, 3, eq, _ffi.FLUX_LLF, precision)
        sv.set_option(_ffi.OPT_PREFETCH, pre)
        sv.project(ic, params)
        sv.set_dt(None)
        sv.run(max_steps=5)
        out.append(sv.get_state())
    np.testing.assert_array_equal(out[0], out[1])
