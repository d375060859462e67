"""The FP64 oracle against golden vectors produced by the reference's own CPU
Euler loops (tests/golden/make_golden.py): tables, geometry, one RHS and a few
RK4 steps.  With ref_sqrtf the oracle mimics the reference's single-precision
square roots and must agree to rounding; as a true FP64 scheme it must agree to
the size of that sqrtf noise."""
import glob
import os

import numpy as np
import pytest

from dgcuda_gb300.mesh import Mesh

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "euler_*.npz")))

# the reference's hard-coded basis table is accurate to ~1e-14 (p<=2), 4e-11
# (p=3), 6e-9 (p=4), 2e-6 (p=5); its 6-point Gauss rule carries 8 digits
TABLE_TOL = {0: 1e-14, 1: 1e-13, 2: 1e-12, 3: 1e-10, 4: 1e-8, 5: 1e-5}
RHS_TOL = {0: 1e-12, 1: 1e-12, 2: 1e-12, 3: 1e-10, 4: 1e-9, 5: 5e-6}


def load(path):
    z = np.load(path)
    m = Mesh(*z["V"], *z["elem_s"], *z["sides"])
    return z, m


def test_golden_present():
    assert len(GOLDEN) >= 8


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_tables_match_reference(path, oracle_mod):
    z, _ = load(path)
    p = int(z["p"])
    T = oracle_mod.tables(p)
    for k in ("r1", "r2", "w", "s1", "w1", "phi", "gx", "gy", "side", "vert"):
        assert np.abs(T[k] - z["ref_" + k]).max() <= TABLE_TOL[p], k


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference(path, oracle_mod):
    orc = oracle_mod
    z, m = load(path)
    p = int(z["p"])
    o = orc.Oracle(m, p, orc.EULER, orc.LLF, 1.4, ref_sqrtf=True)
    g = o.geometry()
    for k in ("J", "xr", "yr", "xs", "ys", "diam", "len", "nx", "ny"):
        np.testing.assert_array_equal(g[k], z["ref_" + k], err_msg=k)
    k = o.rhs(z["c0"], 1.0)
    assert orc.rel_l2(k, z["ref_rhs"]).max() <= RHS_TOL[p]
    c = z["c0"].copy()
    for _ in range(int(z["nsteps"])):
        c = o.step(c, float(z["dt"]))
    assert orc.rel_l2(c, z["ref_c_final"]).max() <= RHS_TOL[p] * 1e-2
    # true FP64 restatement: differs from the reference only by its sqrtf rounding
    o64 = orc.Oracle(m, p, orc.EULER, orc.LLF, 1.4, ref_sqrtf=False)
    assert orc.rel_l2(o64.rhs(z["c0"], 1.0), z["ref_rhs"]).max() <= max(1e-7, RHS_TOL[p])
    lam = o64.max_lambda(z["c0"])
    assert abs(lam - z["ref_lambda"].max()) <= 1e-6 * lam


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_forward_euler_matches_reference(path, oracle_mod):
    """Forward-Euler steps against the reference's eval_rhs_fe loop."""
    orc = oracle_mod
    z, m = load(path)
    p = int(z["p"])
    o = orc.Oracle(m, p, orc.EULER, orc.LLF, 1.4, ref_sqrtf=True)
    o.set_integrator(orc.FE)
    c = z["c0"].copy()
    for _ in range(int(z["nsteps"])):
        c = o.step(c, float(z["dt"]))
    assert orc.rel_l2(c, z["ref_c_fe"]).max() <= RHS_TOL[p] * 1e-2
