"""Tensor-core (tcgen05) known-answer test: a BF16 MMA of small integers with
FP32 accumulation must be exact, with A from shared and from tensor memory."""
import ctypes as C

import numpy as np
import pytest

from dgcuda_gb300 import _ffi

pytestmark = pytest.mark.gpu


def run(variant):
    bad_ss, bad_ts = C.c_int(-1), C.c_int(-1)
    vals = np.zeros((128, 64), dtype=np.float32)
    _ffi.call("dgx_tc_selftest", variant, C.byref(bad_ss), C.byref(bad_ts), vals.ctypes.data_as(C.c_void_p))
    return bad_ss.value, bad_ts.value, vals


def expected():
    m = np.arange(128)[:, None]
    k = np.arange(16)[None, :]
    A = ((3 * m + 5 * k) % 7 - 3).astype(np.float64)
    n = np.arange(32)[:, None]
    B = ((2 * n + k) % 5 - 2).astype(np.float64)
    return A @ B.T


def test_tensor_core_mma_is_exact(gpu):
    bad_ss, bad_ts, vals = run(0)
    ref = expected()
    assert bad_ss == 0, (bad_ss, np.abs(vals[:, :32] - ref).max())
    assert bad_ts == 0, (bad_ts, np.abs(vals[:, 32:] - ref).max())
    np.testing.assert_array_equal(vals[:, :32], ref)
    np.testing.assert_array_equal(vals[:, 32:], ref)


def test_exchanged_descriptor_offsets_are_detected(gpu):
    """The diagnostic variant reads the same operands with LBO and SBO
    exchanged: the product must come out wrong, so the check has teeth."""
    bad_ss, _, _ = run(1)
    assert bad_ss > 0
