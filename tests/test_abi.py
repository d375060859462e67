"""The C ABI without a GPU: the library loads, exports every function that
include/*.h declares, serves the FP64 tables, and rejects malformed meshes on
the host before touching the device."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(dgx_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(native):
    decl = declared_functions()
    assert len(decl) >= 25
    for name in decl:
        assert hasattr(native, name), name
        assert name in _ffi.SIGNATURES, name


def test_version_and_status_strings(native):
    assert native.dgx_version() == 1
    assert native.dgx_status_string(0) == b"ok"
    assert native.dgx_status_string(_ffi.ERR_UNSUPPORTED) == b"unsupported"


@pytest.mark.parametrize("p", range(6))
def test_tables_match_oracle(p, native, oracle_mod):
    from dgcuda_gb300.solver import tables
    A, B = tables(p), oracle_mod.tables(p)
    for k in ("r1", "r2", "w", "s1", "w1", "phi", "gx", "gy", "side", "vert"):
        np.testing.assert_allclose(A[k], B[k], rtol=0, atol=1e-14, err_msg=k)


def test_tables_reject_bad_order(native):
    dims = (C.c_int * 3)()
    nulls = [None] * 10
    assert native.dgx_tables(6, dims, *nulls) == _ffi.ERR_UNSUPPORTED
    assert native.dgx_tables(-1, dims, *nulls) == _ffi.ERR_UNSUPPORTED


def _create(m):
    from dgcuda_gb300.solver import _dp, _ip
    h = C.c_void_p()
    V = [np.ascontiguousarray(a, dtype=np.float64) for a in m.vertices()]
    I = [np.ascontiguousarray(a, dtype=np.int32) for a in m.elem_sides() + m.side_arrays()]
    rc = _ffi.lib().dgx_mesh_create(m.num_elem, m.num_sides, *[_dp(a) for a in V],
                                   *[_ip(a) for a in I], C.byref(h))
    return rc, _ffi.lib().dgx_last_error().decode()


@pytest.mark.parametrize("defect", ["clockwise", "elem_s", "range", "same", "tag"])
def test_mesh_validation_on_host(defect, native):
    m = periodic_square(3, jitter=0.1, seed=1)
    if defect == "clockwise":
        m.V2x[0], m.V3x[0] = m.V3x[0], m.V2x[0]
        m.V2y[0], m.V3y[0] = m.V3y[0], m.V2y[0]
    elif defect == "elem_s":
        m.elem_s1[0], m.elem_s2[0] = m.elem_s2[0], m.elem_s1[0]
    elif defect == "range":
        m.left_elem[2] = m.num_elem
    elif defect == "same":
        m.right_elem[0] = m.left_elem[0]
    elif defect == "tag":
        m.right_elem[0] = -7
    rc, msg = _create(m)
    assert rc == _ffi.ERR_INVALID, msg
    assert msg


def header_constants():
    """Every enumerator `DGX_NAME = value` the headers declare."""
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for body in re.findall(r"enum\s+\w*\s*\{(.*?)\}", text, flags=re.S):
            for name, val in re.findall(r"\b(DGX_[A-Z0-9_]+)\s*=\s*(-?\d+)", body):
                out[name] = int(val)
    return out


def test_binding_constants_match_header():
    """The ctypes binding's constants are the header's enumerators (every one
    the binding names), so Python callers and C callers pass the same codes."""
    hdr = header_constants()
    assert hdr["DGX_IC_LINEAR"] == 8 and hdr["DGX_FP32_COMP"] == 3
    matched = 0
    for name, val in hdr.items():
        short = name[4:]
        if hasattr(_ffi, short):
            assert getattr(_ffi, short) == val, name
            matched += 1
    for short in ("IC_LINEAR", "IC_THREEPOINT", "BC_EXACT", "FP32_COMP", "RK2", "FLUX_LLF", "OPT_HOOK_MATH"):
        assert "DGX_" + short in hdr and hasattr(_ffi, short), short
    assert matched >= 40, matched
