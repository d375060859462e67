"""The BF16x3 tensor-core path (DGX_FP32_BF16X3) against the FP64 oracle and the
plain FP32 path: one RHS, RK4 steps, CFL runs, boundary meshes, conservation,
and the orders and modes it refuses."""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.batch import Batch
from dgcuda_gb300.mesh import dirichlet_square, periodic_square, scramble, tag_boundary
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BF = _ffi.FP32_BF16X3
VORTEX = (5.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0)
WAVE = (0.2, 1.0, 1.0, 1.0, 1.0)
# one RHS: the BF16 hi/lo operands carry 16 of FP32's 24 mantissa bits
# (2^-17 relative), and the element's volume and surface terms nearly cancel,
# which amplifies that relative error in the small net RHS (as FP32 rounding
# is amplified for the FP32 path); states after whole runs stay within 1e-5
RHS_TOL = 5e-4
STATE_TOL = 1e-5


def rel_l2(a, b):
    nv = a.shape[0]
    a = a.reshape(nv, -1)
    b = b.reshape(nv, -1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def f32(c):
    return c.astype(np.float32).astype(np.float64)


def gpu_rhs(sv, c, dt=1.0, t=0.0):
    u = torch.tensor(np.ascontiguousarray(c), dtype=torch.float32, device="cuda")
    k = torch.zeros_like(u)
    sv.rhs_eval(u.data_ptr(), k.data_ptr(), dt, t, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return k.double().cpu().numpy()


def make_case(kind, n=4, seed=0):
    if kind == "vortex":
        return periodic_square(n, lx=10.0, ly=10.0, jitter=0.15, seed=seed), _ffi.EULER, _ffi.IC_VORTEX, VORTEX
    if kind == "wave":
        return periodic_square(n, jitter=0.15, seed=seed), _ffi.EULER, _ffi.IC_DENSITY_WAVE, WAVE
    return (periodic_square(n, jitter=0.15, seed=seed), _ffi.ADVECTION, _ffi.IC_GAUSSIAN,
            (0.4, 0.6, 0.05, 1.0, 1.0))


@pytest.mark.parametrize("flux", [_ffi.FLUX_LLF, _ffi.FLUX_CENTRAL], ids=["llf", "central"])
@pytest.mark.parametrize("kind", ["vortex", "wave", "advection"])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_rhs_matches_oracle(p, kind, flux, gpu, oracle_mod):
    orc = oracle_mod
    m, eq, ic, params = make_case(kind, n=12, seed=p)
    m = scramble(m, seed=p + 20)
    a = (1.0, 0.5)
    o = orc.Oracle(m, p, eq, flux, 1.4, a=a)
    c = f32(o.project(ic, params))
    ref = o.rhs(c, 1.0)
    err = rel_l2(gpu_rhs(Solver(m, p, eq, flux, BF, 1.4, a=a), c), ref).max()
    err32 = rel_l2(gpu_rhs(Solver(m, p, eq, flux, _ffi.FP32, 1.4, a=a), c), ref).max()
    assert err <= RHS_TOL, (err, err32)


@pytest.mark.parametrize("kind,p", [("vortex", 3), ("wave", 3), ("wave", 4), ("vortex", 2), ("advection", 3),
                                    ("advection", 1)])
def test_rk4_cfl_run_matches_oracle(kind, p, gpu, oracle_mod):
    orc = oracle_mod
    m, eq, ic, params = make_case(kind, n=16, seed=p)
    m = scramble(m, seed=p)
    o = orc.Oracle(m, p, eq, orc.LLF, a=(1.0, 0.5))
    c = f32(o.project(ic, params))
    t_end = 0.3 if kind == "vortex" else 0.02
    ref, n, t = o.run(c, t_end)
    sv = Solver(m, p, eq, _ffi.FLUX_LLF, BF, a=(1.0, 0.5))
    sv.set_state(c)
    sv.set_dt(cfl=0.7)
    n2, t2 = sv.run(t_end=t_end)
    assert n2 == n and abs(t2 - t) < 1e-12
    assert rel_l2(sv.get_state(), ref).max() <= STATE_TOL


def test_matches_fp32_path_and_conserves(gpu):
    """BF16x3 and plain FP32 agree to FP32 level after 50 steps; the conserved
    totals drift by no more than FP32 rounding."""
    m = periodic_square(24, jitter=0.15, seed=5)
    out = {}
    for prec in (_ffi.FP32, BF):
        sv = Solver(m, 3, _ffi.EULER, _ffi.FLUX_LLF, prec)
        sv.project(_ffi.IC_DENSITY_WAVE, WAVE)
        tot0 = sv.totals()
        sv.set_dt(cfl=0.7)
        sv.run(max_steps=50)
        out[prec] = (sv.get_state(), np.abs(sv.totals() - tot0) / np.abs(tot0))
    assert rel_l2(out[BF][0], out[_ffi.FP32][0]).max() <= STATE_TOL
    assert out[BF][1].max() <= 1e-6


@pytest.mark.parametrize("p", [2, 3])
def test_boundary_mesh_matches_oracle(p, gpu, oracle_mod):
    orc = oracle_mod
    m = tag_boundary(dirichlet_square(10, lx=10.0, ly=10.0, jitter=0.15, seed=p),
                     lambda x, y: -3 if x < 1e-9 else (-2 if x > 10 - 1e-9 else -1))
    fs = (1.0, 0.5, 0.0, 1.0)
    o = orc.Oracle(m, p, orc.EULER, orc.LLF)
    o.set_boundary(1, 0, fs)
    c = f32(o.project(orc.IC_VORTEX, (5.0, 5.0, 3.0, 0.5, 0.0, 0.0, 0.0)))
    sv = Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, BF)
    sv.set_boundary(_ffi.BC_FREESTREAM, 0, fs)
    assert rel_l2(gpu_rhs(sv, c), o.rhs(c)).max() <= RHS_TOL
    dt = 0.3 * o.cfl_dt(c)
    ref = c.copy()
    for s in range(10):
        ref = o.step(ref, dt, t=s * dt)
    sv.set_state(c)
    sv.set_dt(dt)
    sv.run(max_steps=10)
    assert rel_l2(sv.get_state(), ref).max() <= STATE_TOL


def test_rk2_and_tiles_with_a_ragged_last_tile(gpu, oracle_mod):
    """E not a multiple of the 128-element tile, RK2: the dead lanes of the last
    tile take part in the tensor-memory traffic and write nothing."""
    orc = oracle_mod
    m = scramble(periodic_square(9, jitter=0.1, seed=2), seed=3)   # 162 elements
    o = orc.Oracle(m, 3, orc.EULER, orc.LLF)
    o.set_integrator(orc.RK2)
    c = f32(o.project(orc.IC_DENSITY_WAVE, WAVE))
    ref, n, _ = o.run(c, 0.01)
    sv = Solver(m, 3, _ffi.EULER, _ffi.FLUX_LLF, BF, integrator=_ffi.RK2)
    sv.set_state(c)
    sv.set_dt(cfl=0.7)
    n2, _ = sv.run(t_end=0.01)
    assert n2 == n
    assert rel_l2(sv.get_state(), ref).max() <= STATE_TOL


@pytest.mark.parametrize("p", [0, 5])
def test_orders_outside_1_to_4_are_refused(p, gpu):
    m = periodic_square(4)
    with pytest.raises(_ffi.DgxError) as ei:
        Solver(m, p, _ffi.EULER, _ffi.FLUX_LLF, BF)
    assert ei.value.status == _ffi.ERR_UNSUPPORTED


def test_batches_refuse_bf16x3(gpu):
    m = periodic_square(4)
    with pytest.raises(_ffi.DgxError) as ei:
        Batch([Solver(m, 2, _ffi.EULER, _ffi.FLUX_LLF, BF)])
    assert ei.value.status == _ffi.ERR_UNSUPPORTED
