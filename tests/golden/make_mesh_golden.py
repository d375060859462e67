"""Collect the reference's own Gmsh meshes and the .pmsh files its converter
made from them, as test fixtures.

The reference ships .msh / .pmsh pairs: the Gmsh v2.2 input and the output of
its converter (src/2d/genmesh.py) that its solvers read.  This script stores
the pairs of the current .pmsh format that are small enough to commit, as
text, in tests/golden/reference_meshes.npz; tests/test_meshio_reference.py
converts each .msh and compares with the stored .pmsh byte for byte, and the
GPU tests run the reference's problems on them.

Needs the reference tree, so it runs only where the reference is mounted:

    python tests/golden/make_mesh_golden.py REFERENCE_ROOT   (or set DGX_REFERENCE_ROOT)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# name -> path of the .msh within the reference tree (the .pmsh sits beside it)
PAIRS = {
    "sample": "src/2d/mesh/sample.msh",
    "cylinder": "src/2d/conservation/euler/cylinder/mesh/cylinder.msh",
    "cylinder1": "src/2d/conservation/euler/cylinder/mesh/cylinder1.msh",
    "sv1": "src/2d/conservation/euler/supersonic/mesh/sv1.msh",
}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DGX_REFERENCE_ROOT", "")
    if not root or not os.path.isdir(root):
        raise SystemExit("usage: make_mesh_golden.py REFERENCE_ROOT (or set DGX_REFERENCE_ROOT)")
    out = {}
    for name, rel in PAIRS.items():
        msh = os.path.join(root, rel)
        with open(msh, "rb") as f:
            out[f"{name}_msh"] = np.frombuffer(f.read(), dtype=np.uint8)
        with open(msh[:-4] + ".pmsh", "rb") as f:
            out[f"{name}_pmsh"] = np.frombuffer(f.read(), dtype=np.uint8)
        out[f"{name}_source"] = np.frombuffer(rel.encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "reference_meshes.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_meshes.npz"), sorted(PAIRS))


if __name__ == "__main__":
    main()
