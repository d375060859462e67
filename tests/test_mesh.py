"""Structured periodic mesh generator and scrambler (CPU)."""
import numpy as np
import pytest

from dgcuda_gb300.mesh import periodic_square, scramble


@pytest.mark.parametrize("n", [1, 2, 5])
def test_periodic_square_consistent(n):
    m = periodic_square(n, jitter=0.15 if n > 1 else 0.0, seed=1)
    m.check()
    assert m.num_elem == 2 * n * n and m.num_sides == 3 * n * n
    assert np.all(m.right_elem >= 0)
    assert np.all(m.left_elem != m.right_elem)
    # each element appears exactly three times over all side slots
    counts = np.bincount(np.concatenate([m.left_elem, m.right_elem]), minlength=m.num_elem)
    assert np.all(counts == 3)
    # the two traversals of a side are opposite (CCW elements), up to a period
    V = np.stack(m.vertices()).reshape(3, 2, -1)
    for s in range(m.num_sides):
        L, R, ls, rs = m.left_elem[s], m.right_elem[s], m.left_side[s], m.right_side[s]
        dl = V[(ls + 1) % 3, :, L] - V[ls, :, L]
        dr = V[(rs + 1) % 3, :, R] - V[rs, :, R]
        np.testing.assert_allclose(dl, -dr, atol=1e-12)


def test_jitter_keeps_boundary_and_area():
    m = periodic_square(8, jitter=0.15, seed=3)
    assert abs(m.jacobian().sum() / 2 - 1.0) < 1e-12
    assert m.jacobian().min() > 0


def test_scramble_keeps_mesh_valid():
    m = periodic_square(4, jitter=0.15, seed=3)
    for seed in range(4):
        s = scramble(m, seed=seed)
        s.check()
        assert abs(s.jacobian().sum() - m.jacobian().sum()) < 1e-12


@pytest.mark.parametrize("n,jit,seed", [(1, 0.0, 0), (5, 0.15, 12347), (16, 0.3, 7)])
def test_native_generator_matches_python(n, jit, seed, native):
    import ctypes as C
    from dgcuda_gb300 import _ffi
    m = periodic_square(n, lx=2.0, ly=3.0, x0=-1.0, y0=0.5, jitter=jit, seed=seed)
    E, S = m.num_elem, m.num_sides
    V = np.zeros(6 * E)
    es = np.zeros(3 * E, dtype=np.int32)
    sd = np.zeros(4 * S, dtype=np.int32)
    _ffi.call("dgx_periodic_square_arrays", n, 2.0, 3.0, -1.0, 0.5, jit, seed,
              V.ctypes.data_as(C.POINTER(C.c_double)), es.ctypes.data_as(C.POINTER(C.c_int)),
              sd.ctypes.data_as(C.POINTER(C.c_int)))
    np.testing.assert_array_equal(V.reshape(6, E), np.stack(m.vertices()))
    np.testing.assert_array_equal(es.reshape(3, E), np.stack(m.elem_sides()))
    np.testing.assert_array_equal(sd.reshape(4, S), np.stack(m.side_arrays()))
