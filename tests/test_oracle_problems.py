"""The reference's problem plug-ins in the oracle (cylinder, supersonic vortex,
three-point shock): known-answer tests of their initial states and ghost
states."""
import numpy as np

from dgcuda_gb300.mesh import annulus, dirichlet_square, tag_boundary

SUPERSONIC = (2.25, 1.0125)      # M at the inner arc, A (supersonic.cu:10,32)
THREEPOINT = (0.25, 5.0)         # M, theta in degrees (threepoint.cu:14-15)
CYLINDER = (0.38,)               # M (cylinder.cu:10)


def test_supersonic_vortex_is_steady(oracle_mod):
    """The vortex between the arcs r = 1 and 1.384 is an exact steady state:
    its discrete residual falls with the mesh -- mass and energy at the
    scheme's order, momentum at about h^1.5, the limit of straight sides on
    the curved walls."""
    orc = oracle_mod
    res = []
    for n in (4, 8):
        m = annulus(n, 2 * n, 1.0, 1.384, 0.0, np.pi / 2)
        o = orc.Oracle(m, 2, orc.EULER, orc.LLF)
        o.set_boundary(3, orc.IC_SUPERSONIC, SUPERSONIC)
        c = o.project(orc.IC_SUPERSONIC, SUPERSONIC)
        k = o.rhs(c, 1.0)
        g = o.geometry()
        res.append(np.sqrt(np.sum(k[:, 0, :] ** 2 * g["J"], axis=1)))   # cell averages, L2
    ratio = res[0] / res[1]
    assert ratio[0] > 3.5 and ratio[3] > 3.5, ratio
    assert ratio[1] > 2.5 and ratio[2] > 2.5, ratio


def test_supersonic_initial_state(oracle_mod):
    orc = oracle_mod
    U = orc.ic_eval(orc.IC_SUPERSONIC, SUPERSONIC, 1.0, 0.0)   # on the inner arc at theta = 0
    assert abs(U[0] - 1.0) < 1e-15                                   # rho_i = 1
    assert abs(U[1]) < 1e-15 and abs(U[2] + 2.25) < 1e-15             # speed M, clockwise
    U = orc.ic_eval(orc.IC_SUPERSONIC, SUPERSONIC, 0.0, 1.2)         # on the y axis
    assert U[2] == 0.0 or abs(U[2]) < 1e-15


def test_threepoint_shock_region_is_preserved(oracle_mod):
    """Inside the shock region with shock-state ghosts on every side, the
    uniform shock state is a steady solution: RHS = 0 to rounding."""
    orc = oracle_mod
    m = dirichlet_square(4, lx=0.05, ly=1.0, y0=1.0, jitter=0.1, seed=1)
    m = tag_boundary(m, lambda x, y: -3 if x < 1e-9 else -2)
    o = orc.Oracle(m, 3, orc.EULER, orc.LLF)
    o.set_boundary(3, orc.IC_THREEPOINT, THREEPOINT)
    c = o.project(orc.IC_THREEPOINT, THREEPOINT)
    U = orc.ic_eval(orc.IC_THREEPOINT, THREEPOINT, 0.01, 1.5)
    a = 5.0 * 3.14159 / 180
    np.testing.assert_allclose(U, [1.4, 1.4 * 0.25 * np.cos(a), 1.4 * 0.25 * np.sin(a),
                                   0.5 * 1.4 * 0.25 ** 2 + 1 / 0.4], rtol=1e-15)
    k = o.rhs(c, 1.0) * o.geometry()["J"]     # undo the 1/J of these small elements
    assert np.abs(k).max() < 1e-13


def test_threepoint_reflection_flips_one_component(oracle_mod):
    """threepoint.cu:86-109: with m.n > 0 the x momentum flips, else the y
    momentum; density and energy are kept.  Checked through the wall flux of
    a state at rest in x: only the momentum equations see the wall."""
    orc = oracle_mod
    m = tag_boundary(dirichlet_square(3, jitter=0.0, seed=0), lambda x, y: -1)
    o = orc.Oracle(m, 0, orc.EULER, orc.LLF)
    o.set_boundary(3, orc.IC_THREEPOINT, THREEPOINT)
    c = o.project(orc.IC_CONSTANT, (1.0, 0.0, 0.0, 1.0))
    k = o.rhs(c, 1.0)
    np.testing.assert_allclose(k[0], 0.0, atol=1e-14)   # no mass through the walls
    np.testing.assert_allclose(k[3], 0.0, atol=1e-14)


def test_cylinder_free_stream_through_far_field(oracle_mod):
    """A uniform free stream with free-stream ghosts on the outer circle and
    a wall-free ring gap is steady: no reflecting side, RHS = 0 to rounding."""
    orc = oracle_mod
    m = annulus(3, 24, 0.2, 0.5, cx=0.5, cy=0.5, tag=lambda x, y, w: -3 if x < 0.5 else -2)
    o = orc.Oracle(m, 2, orc.EULER, orc.LLF)
    o.set_boundary(3, orc.IC_CYLINDER, CYLINDER)
    c = o.project(orc.IC_CYLINDER, CYLINDER)
    assert np.abs(o.rhs(c, 1.0)).max() < 1e-11
    U = orc.ic_eval(orc.IC_CYLINDER, CYLINDER, 0.3, 0.7)
    np.testing.assert_allclose(U, [1.4, 1.4 * 0.38, 0.0, 0.5 * 1.4 * 0.38 ** 2 + 2.5], rtol=1e-15)
