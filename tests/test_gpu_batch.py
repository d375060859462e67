"""Batched path: many independent solves of mixed order, equation, size and
precision advanced together by per-class kernels over (solve, tile) work lists
and a CUDA graph.  Each solve must equal the same solve run alone, bit for bit."""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.batch import Batch
from dgcuda_gb300.mesh import periodic_square, scramble
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# (equation, order, n, precision, dt or None for CFL, scrambled)
CASES = [
    (_ffi.ADVECTION, 1, 8, _ffi.FP32, 2e-3, False),
    (_ffi.ADVECTION, 2, 5, _ffi.FP32, 1e-3, True),      # E = 50: rows not 16-byte aligned
    (_ffi.EULER, 1, 6, _ffi.FP32, None, False),
    (_ffi.EULER, 2, 12, _ffi.FP32, None, False),
    (_ffi.EULER, 3, 10, _ffi.FP32, None, True),
    (_ffi.EULER, 3, 4, _ffi.FP32, None, False),
    (_ffi.ADVECTION, 4, 7, _ffi.FP32, 5e-4, False),
    (_ffi.EULER, 4, 5, _ffi.FP32, None, False),
    (_ffi.EULER, 2, 6, _ffi.FP64, None, False),
    (_ffi.EULER, 3, 24, _ffi.FP32, None, False),
]


NCLASSES = len({(c[0], c[1], c[3]) for c in CASES})


def make(case, seed):
    eq, p, n, prec, dt, scr = case
    if eq == _ffi.EULER:
        m = periodic_square(n, lx=10.0, ly=10.0, jitter=0.15, seed=seed)
        ic, params = _ffi.IC_VORTEX, (5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0)
    else:
        m = periodic_square(n, jitter=0.15, seed=seed)
        ic, params = _ffi.IC_GAUSSIAN, (0.3, 0.6, 0.02, 1.0, 1.0)
    if scr:
        m = scramble(m, seed=seed)
    sv = Solver(m, p, eq, _ffi.FLUX_LLF, prec, a=(1.0, 0.7))
    sv.project(ic, params)
    sv.set_dt(dt)
    return sv


def alone_and_batched(steps):
    alone = [make(c, i) for i, c in enumerate(CASES)]
    mixed = [make(c, i) for i, c in enumerate(CASES)]
    for sv in alone:
        sv.run(max_steps=steps)
    return alone, mixed


def test_batch_equals_solves_alone(gpu):
    alone, mixed = alone_and_batched(6)
    b = Batch(mixed)
    info = b.info()
    assert info["classes"] == NCLASSES and info["launches_per_step"] == 1 + 4 * NCLASSES
    b.run(6)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m.get_state(), a.get_state())
        ta, tm = a.time(), m.time()
        assert ta == tm
    assert b.launch_count() == 6 * info["launches_per_step"]


def test_autotune_keeps_results(gpu):
    alone, mixed = alone_and_batched(5)
    b = Batch(mixed)
    b.run(2)
    b.autotune(reps=2)                 # times the live batch, then restores it
    opts = b.class_options()
    assert len(opts) == NCLASSES and all(o["persistent"] in (0, 2, 4) for o in opts)
    b.run(3)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m.get_state(), a.get_state())


def test_batch_rejects_duplicates(gpu):
    sv = make(CASES[0], 0)
    with pytest.raises(_ffi.DgxError):
        Batch([sv, sv])


FP32_CASES = [c for c in CASES if c[3] == _ffi.FP32]


@pytest.mark.parametrize("mode", [2, 3])
def test_fused_launch_equals_solves_alone(mode, gpu):
    """One kernel per RK stage for every class (a step is 5 launches); each
    solve still equals the same solve run alone, bit for bit."""
    alone = [make(c, i) for i, c in enumerate(FP32_CASES)]
    mixed = [make(c, i) for i, c in enumerate(FP32_CASES)]
    for sv in alone:
        sv.run(max_steps=6)
    b = Batch(mixed)
    assert b.fused() == (0, True)
    b.set_fused(mode)
    assert b.fused() == (mode, True)
    info = b.info()
    assert info["launches_per_step"] == 5
    b.run(6)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m.get_state(), a.get_state())
        assert a.time() == m.time()
    assert b.launch_count() == 6 * 5
    # back to the per-class launches mid-run: the same bits again
    b.set_fused(0)
    assert b.info()["launches_per_step"] == 1 + 4 * len({(c[0], c[1]) for c in FP32_CASES})
    for sv in alone:
        sv.run(max_steps=2)
    b.run(2)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m.get_state(), a.get_state())


def test_fused_launch_refused_where_unsupported(gpu):
    """FP64 solves (and meshes with boundary sides) keep the per-class launches."""
    b = Batch([make(c, i) for i, c in enumerate(CASES)])   # includes an FP64 solve
    assert b.fused() == (0, False)
    with pytest.raises(_ffi.DgxError):
        b.set_fused(2)
    with pytest.raises(_ffi.DgxError):
        Batch([make(FP32_CASES[0], 0)]).set_fused(1)        # not a variant


def test_autotune_may_choose_fused(gpu):
    alone = [make(c, i) for i, c in enumerate(FP32_CASES)]
    mixed = [make(c, i) for i, c in enumerate(FP32_CASES)]
    for sv in alone:
        sv.run(max_steps=5)
    b = Batch(mixed)
    b.run(2)
    b.autotune(reps=2)
    mode, avail = b.fused()
    assert avail and mode in (0, 2, 3)
    b.run(3)
    torch.cuda.synchronize()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m.get_state(), a.get_state())
