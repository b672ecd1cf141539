"""Generates the golden fixtures under tests/golden/.

  reference_meshes.npz  vertices / faces / tets parsed from the reference's own
                        resource/cube/cube2.msh, cube4.msh (written by its
                        MeshUtils::createBeamMsh) and resource/general/single.msh.
                        Read from a checkout of the reference given by
                        --reference (default: XPBD_REFERENCE_DIR, else the
                        checkout oracle/ref/Makefile builds from); only this
                        script reads it, the tests use the .npz.
  oracle_trajectories.npz  FP64 oracle runs on a seeded 3x3x3 cube (sequential
                        Gauss-Seidel, Jacobi, coloured Gauss-Seidel; 10 steps,
                        5 iterations) that pin the oracle against regressions.

Run:  python tests/golden/make_golden.py [--reference PATH]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def seeded_cube():
    X, tets, faces = O.grid_mesh(3, 3, 3, 1.0 / 3)
    rng = np.random.default_rng(1234)
    x0 = X + rng.uniform(-5e-3, 5e-3, X.shape)
    return X, tets, faces, x0


def oracle_runs():
    X, tets, faces, x0 = seeded_cube()
    fixed = (X[:, 2] == 0).astype(np.uint8)
    out = {"X": X, "tets": tets, "x0": x0, "fixed": fixed}
    for name, solver in [("gs", O.GAUSS_SEIDEL), ("jacobi", O.JACOBI), ("cgs", O.COLOURED_GS)]:
        o = O.Oracle(X, tets, faces, 4e3, 0.45, 1000.0, dt=1e-3, g=9.81, num_iter=5, solver=solver)
        o.set_positions(x0)
        o.set_fixed(fixed)
        o.time_steps(10, record=True)
        out[f"{name}_x"] = o.positions()
        out[f"{name}_v"] = o.velocities()
        out[f"{name}_lam"] = o.lambdas()
        out[f"{name}_res"] = o.res_history()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    if a.reference is None:
        import subprocess
        a.reference = os.environ.get("XPBD_REFERENCE_DIR") or subprocess.run(
            ["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "print-ref"], capture_output=True,
            text=True).stdout.strip()
    meshes = {}
    for key, rel in [("cube2", "resource/cube/cube2.msh"), ("cube4", "resource/cube/cube4.msh"),
                     ("single", "resource/general/single.msh")]:
        X, F, T = O.read_msh41(os.path.join(a.reference, rel))
        meshes[f"{key}_X"], meshes[f"{key}_faces"], meshes[f"{key}_tets"] = X, F, T
    np.savez_compressed(os.path.join(HERE, "reference_meshes.npz"), **meshes)
    np.savez_compressed(os.path.join(HERE, "oracle_trajectories.npz"), **oracle_runs())
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
