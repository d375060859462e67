"""dgx_conserved_totals_static: the conserved totals computed with no device
allocation (scratch in a static device array), for callers that cannot call
cudaMalloc.  Called through the C ABI and checked against dgx_conserved_totals
on two calls in a row, to relative 1e-12 (the two reductions add the same FP64
terms in different orders).  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square
from dgcuda_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("precision", [_ffi.FP32, _ffi.FP64], ids=["fp32", "fp64"])
def test_static_totals_match_allocating_totals(precision, gpu):
    mesh = periodic_square(96, lx=10.0, ly=10.0, jitter=0.15, seed=21)   # 18,432 elements
    sv = Solver(mesh, 3, _ffi.EULER, _ffi.FLUX_LLF, precision)
    sv.project(_ffi.IC_VORTEX, (5.0, 5.0, 5.0, 1.0, 0.5, 10.0, 10.0))
    sv.set_dt(None)
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    L = _ffi.lib()
    for call in range(2):                       # two calls in a row, state changed between
        if call == 1:
            sv.run(max_steps=3)
        expected = sv.totals()
        torch.cuda.synchronize()
        rc = L.dgx_conserved_totals_static(sv.h, C.c_void_p(sv.state_ptr()), C.c_void_p(out.data_ptr()),
                                           None)
        assert rc == _ffi.OK, L.dgx_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, expected, rtol=TOL, atol=TOL * np.abs(expected).max())


def test_static_totals_reject_null(gpu):
    mesh = periodic_square(4)
    sv = Solver(mesh, 1, _ffi.ADVECTION, _ffi.FLUX_LLF, _ffi.FP32)
    rc = _ffi.lib().dgx_conserved_totals_static(sv.h, C.c_void_p(sv.state_ptr()), None, None)
    assert rc == _ffi.ERR_INVALID
