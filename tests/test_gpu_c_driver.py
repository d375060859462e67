"""The drop-in binding compiled from C: tests/c_driver/dgx_drop_in.c makes the
calls a reference driver makes (dgx_pmsh_read, dgx_mesh_create,
dgx_solver_create, dgx_solver_set_boundary, dgx_project_ic, dgx_set_dt,
dgx_run, dgx_get_state) against include/dgx.h and libdgx.so, with gcc, and
runs the reference's cylinder problem on the reference's own cylinder.pmsh.
Its final state is compared with the FP64 oracle run of the same problem:
relative L2 per conserved variable <= 1e-11 for the FP64 path, <= 1e-5 for
FP32.  The C compilation itself is checked without a GPU as well."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.mesh import read_pmsh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_driver", "dgx_drop_in.c")
GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_meshes.npz")


def build_driver(out_dir):
    from dgcuda_gb300 import build
    lib = build.build()
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = os.path.join(str(out_dir), "dgx_drop_in")
    libdir = os.path.dirname(lib)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-O2", "-I", os.path.join(ROOT, "include"),
                        "-o", exe, SRC, "-L", libdir, "-ldgx", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_compiles(tmp_path, native):
    assert os.path.exists(build_driver(tmp_path))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(_ffi.FP64, 1e-11), (_ffi.FP32, 1e-5)], ids=["fp64", "fp32"])
def test_c_driver_cylinder_matches_oracle(precision, tol, tmp_path, gpu, oracle_mod):
    orc = oracle_mod
    exe = build_driver(tmp_path)
    z = np.load(GOLDEN)
    mesh_path = tmp_path / "cylinder.pmsh"
    mesh_path.write_bytes(z["cylinder_pmsh"].tobytes())
    m = read_pmsh(str(mesh_path))
    p, mach = 2, 0.38
    o = orc.Oracle(m, p, orc.EULER, orc.LLF)
    o.set_boundary(3, orc.IC_CYLINDER, (mach,))
    o.set_integrator(orc.RK2)
    c0 = o.project(orc.IC_CYLINDER, (mach,))
    t_end = 25.5 * o.cfl_dt(c0)
    ref, nref, _ = o.run(c0, t_end=t_end)
    out = tmp_path / "state.bin"
    r = subprocess.run([exe, str(mesh_path), str(p), "1", str(precision), str(_ffi.IC_CYLINDER),
                        str(_ffi.BC_PROBLEM), repr(t_end), str(out), repr(mach)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    steps, nv, np_, E = struct.unpack("<4i", raw[:16])
    (t,) = struct.unpack("<d", raw[16:24])
    c = np.frombuffer(raw[24:], dtype="<f8").reshape(nv, np_, E)
    assert (nv, np_, E) == (4, 6, m.num_elem)
    assert steps == nref and abs(t - t_end) <= 1e-12 * t_end
    err = orc.rel_l2(c, ref)
    assert err.max() <= tol, err
