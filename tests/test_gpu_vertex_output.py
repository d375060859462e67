"""The Gmsh "ST" vertex-value writer (dgx_write_vertex_values), the
reference's output format (src/2d/conservation/main.cu:193-209: one view per
variable, one `ST (x1,y1,0,x2,y2,0,x3,y3,0) {u1,u2,u3};` line per element,
values at `%lf`).  The values are the modal expansion at the element's
vertices, sum_i c_i phi_i(v), checked against the oracle's vertex table to the
format's 6 decimals."""
import re

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import periodic_square, scramble
from dgcuda_gb300.solver import Solver
from oracle import oracle as orc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ST = re.compile(r"ST \(([^)]*)\) \{([^}]*)\};")


def parse(path):
    text = open(path).read()
    assert text.startswith('View "') and text.rstrip().endswith("};")
    xy, u = [], []
    for a, b in ST.findall(text):
        xy.append([float(x) for x in a.split(",")])
        u.append([float(x) for x in b.split(",")])
    return np.array(xy), np.array(u)


@pytest.mark.parametrize("eq,p,ic,params", [
    (_ffi.ADVECTION, 2, _ffi.IC_GAUSSIAN, (0.4, 0.6, 0.05, 1.0, 1.0)),
    (_ffi.EULER, 3, _ffi.IC_VORTEX, (5.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0)),
])
def test_vertex_values_match_expansion(tmp_path, eq, p, ic, params):
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = 10.0 if eq == _ffi.EULER else 1.0
    mesh = scramble(periodic_square(6, lx=L, ly=L, jitter=0.15, seed=9), seed=4)
    sv = Solver(mesh, p, eq, _ffi.FLUX_LLF, _ffi.FP64)
    sv.project(ic, params)
    c = sv.get_state()
    pattern = str(tmp_path / "U%d.msh")
    _ffi.call("dgx_write_vertex_values", sv.h, pattern.encode())
    sv.close()
    vert = orc.tables(p)["vert"]                      # [Np, 3]
    for n in range(c.shape[0]):
        xy, u = parse(pattern % n)
        assert xy.shape == (mesh.num_elem, 9) and u.shape == (mesh.num_elem, 3)
        for v, (vx, vy) in enumerate(((mesh.V1x, mesh.V1y), (mesh.V2x, mesh.V2y), (mesh.V3x, mesh.V3y))):
            np.testing.assert_allclose(xy[:, 3 * v], vx, atol=6e-7)
            np.testing.assert_allclose(xy[:, 3 * v + 1], vy, atol=6e-7)
            assert np.all(xy[:, 3 * v + 2] == 0.0)
        expect = np.einsum("ie,iv->ev", c[n], vert)   # [E, 3]
        np.testing.assert_allclose(u, expect, atol=6e-7)
