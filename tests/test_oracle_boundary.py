"""Boundary ghost states in the oracle (CPU): the reference's own known-answer
idea (src/2d/test_all.cu:275-498) -- with a = (1,1), u = (x - y)^alpha is
steady, so with exact Dirichlet data its projection stays put for alpha <= p --
plus a fluid at rest in a reflecting box and a free stream through inflow and
outflow sides."""
import numpy as np
import pytest

from dgcuda_gb300.mesh import dirichlet_square, tag_boundary


@pytest.mark.parametrize("p,alpha", [(1, 1), (2, 2), (3, 2), (3, 3), (4, 4)])
@pytest.mark.parametrize("flux", [0, 1], ids=["central", "llf"])
def test_polynomial_steady_state(p, alpha, flux, oracle_mod):
    orc = oracle_mod
    m = dirichlet_square(4, jitter=0.15, seed=alpha)
    o = orc.Oracle(m, p, orc.ADVECTION, flux, a=(1.0, 1.0))
    o.set_boundary(2, orc.IC_POLY, (float(alpha),))
    c = o.project(orc.IC_POLY, (float(alpha),))
    k = o.rhs(c, 1.0, t=0.3)
    assert np.abs(k).max() < 1e-10 * max(1.0, np.abs(c).max())
    c1, n, _ = o.run(c, t_end=0.05, dt=0.002)
    np.testing.assert_allclose(c1, c, atol=1e-11)


def test_rest_in_reflecting_box(oracle_mod):
    orc = oracle_mod
    m = dirichlet_square(5, lx=2.0, ly=1.0, jitter=0.1, seed=2)      # all sides reflecting (-1)
    o = orc.Oracle(m, 3, orc.EULER, orc.LLF)
    c = o.project(orc.IC_CONSTANT, (1.2, 0.0, 0.0, 0.8))
    assert np.abs(o.rhs(c)).max() < 1e-11


def test_free_stream_through_inflow_outflow(oracle_mod):
    orc = oracle_mod
    m = tag_boundary(dirichlet_square(5, jitter=0.1, seed=3),
                     lambda x, y: -3 if x < 1e-9 else (-2 if x > 1 - 1e-9 else -1))
    o = orc.Oracle(m, 2, orc.EULER, orc.LLF)
    # the walls are reflecting: flow parallel to them (v = 0) is steady
    o.set_boundary(1, 0, (1.0, 0.5, 0.0, 1.0))
    c = o.project(orc.IC_CONSTANT, (1.0, 0.5, 0.0, 1.0))
    assert np.abs(o.rhs(c)).max() < 1e-11
