"""dgx_conserved_totals_static: the conserved totals computed with no device
allocation (scratch in a static device array), for callers that cannot call
cudaMalloc.  Called through the C ABI and checked against dgx_conserved_totals
on two calls in a row, to relative 1e-12 (the two reductions add the same FP64
terms in different orders), and against the FP64 oracle's totals.  The cases
cover an element count that is a multiple of the 2048-element block chunk and
one that is not (a short last block), advection (one variable) and a mesh of
more than 256 blocks (the final pass's stride loop).  Collected last on
purpose."""
import ctypes as C

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
VORTEX = (5.0, 5.0, 5.0, 1.0, 0.5, 10.0, 10.0)
GAUSS = (0.5, 0.5, 0.01, 1.0, 1.0)


def _static_totals(sv, out):
    L = _ffi.lib()
    torch.cuda.synchronize()
    rc = L.dgx_conserved_totals_static(sv.h, C.c_void_p(sv.state_ptr()), C.c_void_p(out.data_ptr()), None)
    assert rc == _ffi.OK, L.dgx_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()[: sv.shape[0]].copy()


CASES = [
    # (mesh n, domain side, order, equation, initial condition, its parameters)
    (96, 10.0, 3, _ffi.EULER, _ffi.IC_VORTEX, VORTEX),       # 18,432 = 9 x 2048 elements
    (97, 10.0, 2, _ffi.EULER, _ffi.IC_VORTEX, VORTEX),       # 18,818: a short last block
    (97, 1.0, 2, _ffi.ADVECTION, _ffi.IC_GAUSSIAN, GAUSS),   # one variable
    (520, 1.0, 1, _ffi.ADVECTION, _ffi.IC_GAUSSIAN, GAUSS),  # 540,800: 265 blocks
]


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
@pytest.mark.parametrize("case", CASES, ids=["euler-96", "euler-97", "advec-97", "advec-520"])
def test_static_totals_match_allocating_totals(case, precision, gpu, oracle_mod):
    n, lx, p, eq, ic, params = case
    mesh = periodic_square(n, lx=lx, ly=lx, jitter=0.15, seed=21)
    sv = Solver(mesh, p, eq, _ffi.FLUX_LLF, precision)
    sv.project(ic, params)
    if eq == _ffi.EULER:
        sv.set_dt(None)
    else:
        sv.set_dt(0.1 / n / 2.0 / (2 * p + 1))
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    before = sv.launch_count()
    for call in range(2):                       # two calls in a row, state changed between
        if call == 1:
            sv.run(max_steps=3)
        expected = sv.totals()
        got = _static_totals(sv, out)
        np.testing.assert_allclose(got, expected, rtol=TOL, atol=TOL * np.abs(expected).max())
        # the oracle's totals of the same coefficients (FP64 restatement)
        o = oracle_mod.Oracle(mesh, p, oracle_mod.EULER if eq == _ffi.EULER else oracle_mod.ADVECTION,
                              oracle_mod.LLF)
        ref = o.totals(sv.get_state())
        np.testing.assert_allclose(got, ref, rtol=TOL, atol=TOL * np.abs(ref).max())
    # two totals calls of each kind, three steps: the static variant's launches count
    assert sv.launch_count() > before


def test_static_totals_reject_null(gpu):
    mesh = periodic_square(4)
    sv = Solver(mesh, 1, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP32)
    rc = _ffi.lib().dgx_conserved_totals_static(sv.h, C.c_void_p(sv.state_ptr()), None, None)
    assert rc == _ffi.ERR_INVALID


def test_static_totals_count_launches(gpu):
    mesh = periodic_square(8)
    sv = Solver(mesh, 1, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP32)
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    before = sv.launch_count()
    _static_totals(sv, out)
    assert sv.launch_count() == before + 2
