"""Generate golden vectors from the reference's own CPU Euler loops.

Runs ``oracle/_ref/ref_euler`` (oracle/ref_harness.c compiled against the
reference's src/2d/conservation/euler/cpu sources by ``make -C oracle ref``) on
small seeded periodic meshes and stores, per case, the inputs (mesh arrays,
order, initial coefficients, dt, step count) and the reference's outputs:
basis and quadrature tables, geometric factors, cell wave speeds, one RHS
evaluation with dt = 1, the state after a few fixed-dt RK4 steps and the state
after as many forward-Euler steps from the same start.

Needs the reference tree, so it runs only where the reference is mounted:

    python tests/golden/make_golden.py [/path/to/reference]

The fixtures are committed; tests read them without the reference.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dgcuda_gb300.mesh import periodic_square, scramble  # noqa: E402
from oracle import oracle as orc  # noqa: E402

CASES = [
    # name, mesh builder, p, ic, params, dt, nsteps
    ("wave_p0", lambda: periodic_square(4, jitter=0.15, seed=11), 0, orc.IC_DENSITY_WAVE,
     (0.2, 1.0, 1.0, 1.0, 1.0), 2e-3, 3),
    ("wave_p1", lambda: periodic_square(4, jitter=0.15, seed=11), 1, orc.IC_DENSITY_WAVE,
     (0.2, 1.0, 1.0, 1.0, 1.0), 2e-3, 3),
    ("wave_p2", lambda: periodic_square(4, jitter=0.15, seed=12), 2, orc.IC_DENSITY_WAVE,
     (0.2, 1.0, 1.0, 1.0, 1.0), 1e-3, 3),
    ("wave_p3", lambda: periodic_square(4, jitter=0.15, seed=13), 3, orc.IC_DENSITY_WAVE,
     (0.2, 1.0, 1.0, 1.0, 1.0), 1e-3, 3),
    ("vortex_p3", lambda: periodic_square(4, lx=10.0, ly=10.0, jitter=0.15, seed=14), 3,
     orc.IC_VORTEX, (5.0, 5.0, 5.0, 1.0, 0.0, 10.0, 10.0), 1e-2, 3),
    ("wave_p4", lambda: periodic_square(4, jitter=0.15, seed=15), 4, orc.IC_DENSITY_WAVE,
     (0.2, 1.0, 1.0, 1.0, 1.0), 5e-4, 3),
    ("wave_p5", lambda: periodic_square(3, jitter=0.15, seed=16), 5, orc.IC_DENSITY_WAVE,
     (0.2, 1.0, 1.0, 1.0, 1.0), 4e-4, 2),
    ("scrambled_vortex_p2", lambda: scramble(periodic_square(3, lx=10.0, ly=10.0, jitter=0.15,
                                                             seed=17), seed=3), 2,
     orc.IC_VORTEX, (5.0, 5.0, 3.0, 1.0, 0.5, 10.0, 10.0), 2e-2, 3),
    ("scrambled_wave_p3", lambda: scramble(periodic_square(3, jitter=0.15, seed=18), seed=4), 3,
     orc.IC_DENSITY_WAVE, (0.2, 1.0, -0.5, 1.0, 1.0), 1e-3, 3),
]


def run_case(ref_bin, name, build, p, ic, params, dt, nsteps):
    mesh = build()
    E, S = mesh.num_elem, mesh.num_sides
    o = orc.Oracle(mesh, p, orc.EULER, orc.LLF, 1.4)
    c0 = o.project(ic, params)
    npm = orc.num_modes(p)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            # nsteps RK4 steps, then as many forward-Euler steps from c0
            np.array([E, S, p, nsteps, nsteps, 0, 0, 0], dtype=np.int32).tofile(f)
            np.array([dt], dtype=np.float64).tofile(f)
            for a in mesh.vertices():
                a.astype(np.float64).tofile(f)
            for a in mesh.elem_sides():
                a.astype(np.int32).tofile(f)
            for a in mesh.side_arrays():
                a.astype(np.int32).tofile(f)
            c0.astype(np.float64).tofile(f)
        subprocess.run([ref_bin, fin, fout], check=True, stdout=subprocess.DEVNULL)
        raw = open(fout, "rb").read()
    dims = np.frombuffer(raw[:16], dtype=np.int32)
    np_, nq, nq1 = (int(x) for x in dims[:3])
    assert np_ == npm
    off = 16
    out = {}

    def take(key, n, shape=None):
        nonlocal off
        a = np.frombuffer(raw[off:off + 8 * n], dtype=np.float64).copy()
        off += 8 * n
        out[key] = a.reshape(shape) if shape else a

    take("r1", nq); take("r2", nq); take("w", nq); take("s1", nq1); take("w1", nq1)
    take("phi", np_ * nq, (np_, nq)); take("gx", np_ * nq, (np_, nq)); take("gy", np_ * nq, (np_, nq))
    take("side", 3 * np_ * nq1, (3, np_, nq1)); take("vert", 3 * np_, (np_, 3))
    for k in ("J", "xr", "yr", "xs", "ys", "diam"):
        take(k, E)
    for k in ("len", "nx", "ny"):
        take(k, S)
    take("lambda", E)
    take("rhs", 4 * np_ * E, (4, np_, E))
    take("c_final", 4 * np_ * E, (4, np_, E))
    take("c_fe", 4 * np_ * E, (4, np_, E))
    assert off == len(raw)
    arrays = dict(
        p=np.int32(p), nsteps=np.int32(nsteps), dt=np.float64(dt), ic=np.int32(ic),
        params=np.array(params, dtype=np.float64),
        V=np.stack(mesh.vertices()), elem_s=np.stack(mesh.elem_sides()),
        sides=np.stack(mesh.side_arrays()), c0=c0, **{"ref_" + k: v for k, v in out.items()})
    np.savez_compressed(os.path.join(HERE, f"euler_{name}.npz"), **arrays)
    return name


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else orc.env_reference_root()
    if not ref_root:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT (or set DGX_REFERENCE_ROOT)")
    ref_bin = orc.build_ref(ref_root)
    if ref_bin is None:
        raise SystemExit(f"reference tree not found at {ref_root}")
    for case in CASES:
        print("golden:", run_case(ref_bin, *case))


if __name__ == "__main__":
    main()
