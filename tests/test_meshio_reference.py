"""Mesh I/O pinned to the reference's own files (CPU).

The reference ships Gmsh .msh files beside the .pmsh files its converter
(src/2d/genmesh.py) made from them.  tests/golden/reference_meshes.npz holds
four such pairs (tests/golden/make_mesh_golden.py); every current-format pair
of the reference tree is checked as well when DGX_REFERENCE_ROOT names the
tree.  For each pair:

* gmsh_to_pmsh(.msh) is the reference's .pmsh byte for byte (side order,
  left/right elements, side numbers, six-decimal coordinates);
* the Python reader and the native reader (dgx_pmsh_read) read the .pmsh to
  the same arrays;
* for the pairs that are valid meshes (counter-clockwise triangles, every
  boundary line tagged), read_gmsh gives the .pmsh's index arrays exactly and
  its coordinates to the file's six decimals.

The reference's .pmsh files in the older element-only layout (uniform, simple,
complex, canonical, crazysimple, supersimple: six coordinates per line, no
side table) predate the reader of its solvers (src/2d/conservation/conserv.cu:
118-192) and are not compared.  cyl16.msh is in the Gmsh v1 layout, which the
reference's converter cannot read (its cyl16.pmsh is empty).
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import gmsh_to_pmsh, read_gmsh, read_pmsh

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_meshes.npz")
VALID = {"cylinder", "cylinder1", "sv1", "sv1refined", "sv1refined1", "sv1refined2"}
OLD_LAYOUT = {"uniform", "simple", "complex", "canonical", "crazysimple", "supersimple"}


def _fixture_pairs():
    z = np.load(GOLDEN)
    names = sorted({k.rsplit("_", 1)[0] for k in z.files})
    return [(n, z[f"{n}_msh"].tobytes().decode(), z[f"{n}_pmsh"].tobytes().decode()) for n in names]


def _tree_pairs():
    root = os.environ.get("DGX_REFERENCE_ROOT", "")
    if not root or not os.path.isdir(root):
        return []
    out = []
    for msh in sorted(glob.glob(os.path.join(root, "src", "2d", "**", "*.msh"), recursive=True)):
        name = os.path.basename(msh)[:-4]
        pm = msh[:-4] + ".pmsh"
        if name in OLD_LAYOUT or not os.path.exists(pm) or os.path.getsize(pm) == 0:
            continue
        out.append((name, open(msh).read(), open(pm).read()))
    return out


FIXTURES = _fixture_pairs()


def _native_read(path):
    E, S = C.c_int(), C.c_int()
    _ffi.call("dgx_pmsh_info", path.encode(), C.byref(E), C.byref(S))
    V = np.zeros(6 * E.value)
    es = np.zeros(3 * E.value, dtype=np.int32)
    sd = np.zeros(4 * S.value, dtype=np.int32)
    _ffi.call("dgx_pmsh_read", path.encode(), V.ctypes.data_as(C.POINTER(C.c_double)),
              es.ctypes.data_as(C.POINTER(C.c_int)), sd.ctypes.data_as(C.POINTER(C.c_int)))
    return V.reshape(6, -1), es.reshape(3, -1), sd.reshape(4, -1)


def _check_pair(name, msh, pmsh, tmp_path):
    assert gmsh_to_pmsh(msh) == pmsh, f"{name}: the converted file differs from the reference's"
    p = str(tmp_path / f"{name}.pmsh")
    with open(p, "w") as f:
        f.write(pmsh)
    r = read_pmsh(p)
    V, es, sd = _native_read(p)
    np.testing.assert_array_equal(V, np.stack(r.vertices()))
    np.testing.assert_array_equal(es, np.stack(r.elem_sides()))
    np.testing.assert_array_equal(sd, np.stack(r.side_arrays()))
    if name in VALID:
        r.check()
        m = read_gmsh(msh)
        for a, b in zip(m.elem_sides() + m.side_arrays(), r.elem_sides() + r.side_arrays()):
            np.testing.assert_array_equal(a, b)
        for a, b in zip(m.vertices(), r.vertices()):
            assert np.abs(a - b).max() <= 5.000001e-7
    return r


def test_fixtures_present():
    assert {n for n, _, _ in FIXTURES} == {"sample", "cylinder", "cylinder1", "sv1"}


@pytest.mark.parametrize("name,msh,pmsh", FIXTURES, ids=[f[0] for f in FIXTURES])
def test_converter_matches_reference_files(name, msh, pmsh, tmp_path, native):
    r = _check_pair(name, msh, pmsh, tmp_path)
    if name == "cylinder":
        # the cylinder problem's mesh: boundary sides first, walls (-1) then
        # the far field (-2)
        re = r.right_elem
        nb = int((re < 0).sum())
        assert nb > 0 and np.all(re[:nb] < 0) and np.all(np.diff(re[:nb]) <= 0)
        assert set(re[:nb].tolist()) == {-1, -2}


def test_sample_mesh_is_not_solvable_as_written():
    """sample.msh tags its outer lines with physical group 0, which the
    reference's converter does not know: its .pmsh leaves element 0 as the
    right neighbour of those sides.  read_gmsh makes them reflecting instead."""
    name, msh, pmsh = next(f for f in FIXTURES if f[0] == "sample")
    lines = pmsh.splitlines()
    E = int(lines[0])
    sides = np.array([ln.split()[4:] for ln in lines[2 + E:]], dtype=int)
    assert np.all(sides[:, 1] >= 0)            # the reference's file has no boundary sides
    m = read_gmsh(msh)
    nb = int((m.right_elem < 0).sum())
    assert nb == 8 and np.all(m.right_elem[:nb] == -1)
    m.check()


@pytest.mark.skipif(not _tree_pairs(), reason="DGX_REFERENCE_ROOT does not name the reference tree")
def test_every_reference_pair(tmp_path, native):
    pairs = _tree_pairs()
    assert len(pairs) >= 8
    for name, msh, pmsh in pairs:
        _check_pair(name, msh, pmsh, tmp_path)
