"""TEST INFRASTRUCTURE ONLY: the reference's own CUDA solvers as test references and a
reported baseline, never as the product path.

`oracle/_ref/ref_gpu_euler` and `ref_gpu_advec` are built by `make -C oracle
ref-gpu` from the reference's unmodified sources (src/2d/conservation,
src/2d/2dadvec and src/2d/{time_integrator,quadrature,basis}.cu, from the
reference tree or the copy `make -C oracle ref-src` installs under
baseline/_ref) with `ref_gpu_harness.cu` as their problem file and driver.
`run` hands the Euler solver a mesh and an initial state and lets the
reference's time_integrate_rk4 (src/2d/conservation/time_integrator.cu:221-434),
or time_integrate_rk2 (:466-614), advance to t_end with its CFL rule: on
periodic meshes with the harness's own hooks, or with the boundary hooks of the
reference's cylinder (src/2d/conservation/euler/cylinder/cylinder.cu),
supersonic-vortex (euler/supersonic/supersonic.cu) or three-point shock
(euler/threepoint/threepoint.cu) problem file, compiled in (`problem`);
`run_advection` lets the advection solver's time_integrate_rk4
(src/2d/time_integrator.cu:89-315) take a number of steps of a fixed dt
(a = (1,1), central flux).  Both return the state, the steps taken and the
time.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "ref_gpu_euler")
BIN_ADVEC = os.path.join(HERE, "_ref", "ref_gpu_advec")
BIN_PROBLEM = {"cylinder": os.path.join(HERE, "_ref", "ref_gpu_cylinder"),
               "supersonic": os.path.join(HERE, "_ref", "ref_gpu_supersonic"),
               "threepoint": os.path.join(HERE, "_ref", "ref_gpu_threepoint")}


def build() -> str | None:
    """Build the harnesses if their sources are at hand; the Euler binary's path
    or None."""
    bins = [BIN, BIN_ADVEC] + list(BIN_PROBLEM.values())
    if not all(os.path.exists(b) for b in bins):
        r = subprocess.run(["make", "-s", "-j4", "-C", HERE, "ref-gpu"], capture_output=True, text=True)
        if r.returncode != 0:
            return None
    return BIN if all(os.path.exists(b) for b in bins) else None


def run(mesh, order: int, c0: np.ndarray, t_end: float, timeout: float = 900.0, problem: str | None = None,
        rk2: bool = False) -> dict:
    """Advance the Euler state c0 (layout c[4][Np][E], FP64) on `mesh` (a
    dgcuda_gb300.mesh.Mesh) to t_end with the reference's solver: periodic
    meshes with problem None, else boundary sides with the hooks of the
    reference's "cylinder", "supersonic" or "threepoint" problem file; RK4, or
    RK2 with rk2."""
    binary = BIN if problem is None else BIN_PROBLEM[problem]
    return _run(binary, mesh, order, c0, 4, 0, t_end, timeout, int(bool(rk2)))


def run_advection(mesh, order: int, c0: np.ndarray, dt: float, steps: int, timeout: float = 900.0) -> dict:
    """`steps` RK4 steps of dt of the advection state c0 (c[Np][E], FP64) on
    `mesh` with the reference's advection solver (a = (1,1)): periodic, or
    with boundary sides tagged -1, whose ghost value is the reference's exact
    data x - 2t + y (2dadvec_kernels.cu:184-186) at t = the step's start."""
    return _run(BIN_ADVEC, mesh, order, c0, 1, int(steps), dt, timeout, 0)


def _run(binary, mesh, order, c0, nv, steps, t_in, timeout, rk2):
    if build() is None:
        raise RuntimeError("the reference's CUDA solvers are not built (no reference sources)")
    binp = binary
    E, S = mesh.num_elem, mesh.num_sides
    npm = (order + 1) * (order + 2) // 2
    c0 = np.ascontiguousarray(c0, dtype=np.float64).reshape(-1)
    if c0.size != nv * npm * E:
        raise ValueError(f"c0 must hold {nv} * Np * E values")
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<6i", E, S, order, steps, rk2, 0))
            f.write(struct.pack("<d", float(t_in)))
            for a in mesh.vertices():
                f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
            for a in mesh.elem_sides():
                f.write(np.ascontiguousarray(a, dtype="<i4").tobytes())
            for a in mesh.side_arrays():
                f.write(np.ascontiguousarray(a, dtype="<i4").tobytes())
            f.write(c0.astype("<f8").tobytes())
        r = subprocess.run([binp, fin, fout], capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference solver failed ({r.returncode}): {r.stderr.strip()[-400:]}")
        with open(fout, "rb") as f:
            steps, _ = struct.unpack("<2i", f.read(8))
            secs, min_r = struct.unpack("<2d", f.read(16))
            c = np.frombuffer(f.read(), dtype="<f8").copy()
    if c.size != c0.size:
        raise RuntimeError("reference solver wrote a short state")
    return {"state": c, "steps": steps, "seconds": secs, "min_r": min_r}
