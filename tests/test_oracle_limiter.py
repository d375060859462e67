"""The p = 1 slope limiter in the oracle: its defining bound, conservation,
idempotence, and its effect on a step profile."""
import numpy as np
import pytest

from dgcuda_gb300.mesh import dirichlet_square, periodic_square, scramble


def side_values(o, c):
    """Traces at the 6 side Gauss points of every element: [nv, E, 6]."""
    from oracle import oracle as orc
    side = orc.tables(o.p)["side"]                     # [3, np, nq1]
    vals = np.einsum("vie,kij->vekj", c, side)         # [nv, E, 3, 2]
    return vals.reshape(c.shape[0], c.shape[2], 6)


def neighbour_range(m, c, phi0):
    E = m.num_elem
    es = np.stack(m.elem_sides())                      # [3, E]
    le, re = m.left_elem[es], m.right_elem[es]
    e = np.arange(E)[None, :]
    nb = np.where(le == e, re, le)
    nb = np.where(nb >= 0, nb, e)
    avg = c[:, 0, :] * phi0                            # [nv, E]
    allv = np.concatenate([avg[:, None, :], avg[:, nb]], axis=1)   # [nv, 4, E]
    return allv.min(axis=1), allv.max(axis=1), avg


def step_state(o, m):
    """A square pulse projected onto p = 1 (discontinuous data)."""
    from oracle import oracle as orc
    c = o.project(orc.IC_GAUSSIAN, (0.5, 0.5, 0.02, 0.0, 0.0))
    cx, cy = m.centroids()
    c[0, 0, :] = np.where((np.abs(cx - 0.5) < 0.2) & (np.abs(cy - 0.5) < 0.2), 1.0, 0.0) / np.sqrt(2.0)
    return c


@pytest.mark.parametrize("mesh", ["periodic", "boundary"])
def test_limited_traces_stay_in_the_neighbour_range(mesh, oracle_mod):
    orc = oracle_mod
    m = periodic_square(10, jitter=0.2, seed=3) if mesh == "periodic" else dirichlet_square(10, jitter=0.2, seed=3)
    m = scramble(m, seed=5)
    o = orc.Oracle(m, 1, orc.ADVECTION, orc.LLF)
    c = step_state(o, m)
    c[0, 1:, :] += 0.3 * np.sin(np.arange(m.num_elem))[None, :]   # slopes of every size and sign
    cl = o.limit(c)
    phi0 = orc.tables(1)["phi"][0, 0]
    lo, hi, avg = neighbour_range(m, c, phi0)
    tv = side_values(o, cl)
    assert np.all(tv >= lo[:, :, None] - 1e-12) and np.all(tv <= hi[:, :, None] + 1e-12)
    np.testing.assert_array_equal(cl[:, 0, :], c[:, 0, :])          # cell averages kept
    assert np.abs(cl - c).max() > 0.1                              # it did limit
    np.testing.assert_allclose(o.limit(cl), cl, rtol=0, atol=1e-14)   # idempotent


def test_smooth_and_constant_states(oracle_mod):
    orc = oracle_mod
    m = periodic_square(32, jitter=0.1, seed=2)
    o = orc.Oracle(m, 1, orc.EULER, orc.LLF)
    c = o.project(orc.IC_CONSTANT, (1.0, 0.3, -0.2, 1.0))
    np.testing.assert_array_equal(o.limit(c), c)
    # a resolved smooth wave is limited only near its extrema: most slopes
    # survive intact
    c = o.project(orc.IC_DENSITY_WAVE, (0.2, 1.0, 1.0, 1.0, 1.0))
    cl = o.limit(c)
    untouched = np.all(cl[0, 1:, :] == c[0, 1:, :], axis=0)
    assert untouched.mean() > 0.5


def test_limited_step_profile_has_smaller_overshoot(oracle_mod):
    orc = oracle_mod
    m = periodic_square(16, jitter=0.1, seed=4)
    res = {}
    for on in (False, True):
        o = orc.Oracle(m, 1, orc.ADVECTION, orc.LLF, a=(1.0, 0.5))
        o.set_limiter(on)
        c = step_state(o, m)
        if on:
            c = o.limit(c)
        out, _, _ = o.run(c, 0.1, cfl=0.3)
        avg = out[0, 0, :] * np.sqrt(2.0)
        res[on] = (avg.max() - 1.0, -avg.min())
    assert max(res[True]) < max(res[False]), res
    assert max(res[True]) < 0.05, res


def test_limiter_needs_p1(oracle_mod):
    orc = oracle_mod
    o = orc.Oracle(periodic_square(3), 2, orc.ADVECTION, orc.LLF)
    with pytest.raises(ValueError):
        o.set_limiter(True)
    with pytest.raises(ValueError):
        o.limit(np.zeros(o.shape))
