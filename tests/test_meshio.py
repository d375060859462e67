"""Mesh file formats: the reference's .pmsh (native and Python readers and
writers agree), and Gmsh v2.2 .msh conversion (CPU)."""
import ctypes as C

import numpy as np

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square, read_gmsh, read_pmsh, scramble, write_pmsh


def test_pmsh_round_trip_python_and_native(tmp_path, native):
    m = scramble(periodic_square(5, lx=2.0, jitter=0.2, seed=3), seed=1)
    p = str(tmp_path / "m.pmsh")
    write_pmsh(m, p)
    r = read_pmsh(p)
    for a, b in zip(m.vertices() + m.elem_sides() + m.side_arrays(),
                    r.vertices() + r.elem_sides() + r.side_arrays()):
        np.testing.assert_array_equal(a, b)
    E, S = C.c_int(), C.c_int()
    _ffi.call("dgx_pmsh_info", p.encode(), C.byref(E), C.byref(S))
    assert (E.value, S.value) == (m.num_elem, m.num_sides)
    V = np.zeros(6 * E.value)
    es = np.zeros(3 * E.value, dtype=np.int32)
    sd = np.zeros(4 * S.value, dtype=np.int32)
    _ffi.call("dgx_pmsh_read", p.encode(), V.ctypes.data_as(C.POINTER(C.c_double)),
              es.ctypes.data_as(C.POINTER(C.c_int)), sd.ctypes.data_as(C.POINTER(C.c_int)))
    np.testing.assert_array_equal(V.reshape(6, -1), np.stack(m.vertices()))
    np.testing.assert_array_equal(sd.reshape(4, -1), np.stack(m.side_arrays()))
    q = str(tmp_path / "n.pmsh")
    _ffi.call("dgx_pmsh_write", q.encode(), E.value, S.value, V.ctypes.data_as(C.POINTER(C.c_double)),
              es.ctypes.data_as(C.POINTER(C.c_int)), sd.ctypes.data_as(C.POINTER(C.c_int)))
    r2 = read_pmsh(q)
    for a, b in zip(m.vertices() + m.elem_sides() + m.side_arrays(),
                    r2.vertices() + r2.elem_sides() + r2.side_arrays()):
        np.testing.assert_array_equal(a, b)


def test_pmsh_reader_rejects_short_lines(tmp_path, native):
    p = tmp_path / "bad.pmsh"
    p.write_text("1\n0 0 1 0 0 1 0 1\n")
    E, S = C.c_int(), C.c_int()
    assert _ffi.lib().dgx_pmsh_info(str(p).encode(), C.byref(E), C.byref(S)) == _ffi.ERR_INVALID


SQUARE_MSH = """$MeshFormat
2.2 0 8
$EndMeshFormat
$Nodes
5
1 0 0 0
2 1 0 0
3 1 1 0
4 0 1 0
5 0.5 0.5 0
$Elements
8
1 1 2 10000 1 1 2
2 1 2 20000 2 2 3
3 1 2 30000 3 3 4
4 1 2 10000 4 4 1
5 2 2 1 1 1 2 5
6 2 2 1 1 2 3 5
7 2 2 1 1 3 4 5
8 2 2 1 1 1 5 4
$EndElements
"""


def test_gmsh_conversion():
    m = read_gmsh(SQUARE_MSH)
    assert m.num_elem == 4 and m.num_sides == 8
    assert np.all(m.jacobian() > 0)                     # the clockwise triangle 8 was reordered
    # boundary sides first, sorted -1 (two), -2, -3
    assert list(m.right_elem[:4]) == [-1, -1, -2, -3]
    assert np.all(m.right_elem[4:] >= 0)
    assert abs(m.jacobian().sum() / 2 - 1.0) < 1e-15
