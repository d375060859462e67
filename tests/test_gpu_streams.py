"""Several solves driven at once through the C ABI on their own streams, each
step with its state copied in from pinned host memory and back out
(dgx_set_state_f32, dgx_step, dgx_get_state_f32): the pattern that overlaps
one solve's host copies with another's step.  The solvers share only the
read-only basis tables, so each solve must equal the same solve stepped alone
on one stream, bit for bit, and the host copy after the last step must hold
its final state."""
import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

VORTEX = (5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0)
GAUSS = (0.3, 0.6, 0.02, 1.0, 1.0)
# (equation, order, mesh n, precision): mixed orders, equations and precisions in flight together
CASES = [
    (_ffi.EULER, 3, 40, _ffi.FP32),
    (_ffi.EULER, 2, 33, _ffi.FP32),
    (_ffi.ADVECTION, 4, 21, _ffi.FP32),
    (_ffi.EULER, 4, 17, _ffi.FP32_COMP),
    (_ffi.EULER, 1, 29, _ffi.FP64),
]
STEPS = 12


def make(case, seed):
    eq, p, n, prec = case
    if eq == _ffi.EULER:
        m = periodic_square(n, lx=10.0, ly=10.0, jitter=0.15, seed=seed)
        ic, params = _ffi.IC_VORTEX, VORTEX
    else:
        m = periodic_square(n, jitter=0.15, seed=seed)
        ic, params = _ffi.IC_GAUSSIAN, GAUSS
    sv = Solver(m, p, eq, _ffi.FLUX_LLF, prec, a=(1.0, 0.7))
    sv.project(ic, params)
    sv.set_dt(None if eq == _ffi.EULER else 0.2 / n / (2 * p + 1))
    return sv


def pinned_state(sv):
    h = torch.empty(int(np.prod(sv.shape)), dtype=torch.float32, pin_memory=True)
    sv.get_state_f32(h.numpy(), 0)
    torch.cuda.synchronize()
    return h


def step_with_copies(sv, host, stream):
    sh = stream.cuda_stream
    sv.set_state_f32(host.numpy(), sh)
    sv.step(sh)
    sv.get_state_f32(host.numpy(), sh)


def test_solves_on_streams_equal_solves_alone(gpu):
    # alone: one solve at a time on one stream, the same host round trip every step
    alone = []
    s0 = torch.cuda.Stream()
    for k, case in enumerate(CASES):
        sv = make(case, 40 + k)
        h = pinned_state(sv)
        for _ in range(STEPS):
            step_with_copies(sv, h, s0)
        torch.cuda.synchronize()
        alone.append((sv.get_state(), h.numpy().copy()))
        sv.close()

    # in flight together: every solve on its own stream, the steps interleaved
    svs = [make(c, 40 + k) for k, c in enumerate(CASES)]
    streams = [torch.cuda.Stream() for _ in svs]
    hosts = [pinned_state(sv) for sv in svs]
    for _ in range(STEPS):
        for sv, h, st in zip(svs, hosts, streams):
            step_with_copies(sv, h, st)
    torch.cuda.synchronize()
    for k, (sv, h) in enumerate(zip(svs, hosts)):
        c_alone, h_alone = alone[k]
        np.testing.assert_array_equal(sv.get_state(), c_alone, err_msg=f"case {k}")
        np.testing.assert_array_equal(h.numpy(), h_alone, err_msg=f"case {k} host copy")
        # the host copy after the last step is the final state rounded to FP32
        # (a compensated solve's copy is its FP32 part, without the low part)
        if CASES[k][3] != _ffi.FP32_COMP:
            np.testing.assert_array_equal(h.numpy().reshape(sv.shape), sv.get_state().astype(np.float32))
        assert np.isfinite(h.numpy()).all()
        sv.close()


def test_round_trip_keeps_fp32_state(gpu):
    """dgx_set_state_f32 of what dgx_get_state_f32 returned leaves an FP32
    solve's state bitwise unchanged, so stepping with the host round trip
    equals stepping without it."""
    a, b = make(CASES[0], 7), make(CASES[0], 7)
    h = pinned_state(b)
    st = torch.cuda.Stream()
    for _ in range(STEPS):
        step_with_copies(b, h, st)
    a.run(max_steps=STEPS)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(a.get_state(), b.get_state())
    a.close()
    b.close()
