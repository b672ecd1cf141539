"""Writes tests/golden/reference_kat.npz: inputs and outputs of the
reference's own constraint and projector code, run through
oracle/_ref/libref_kat.so (built from the reference's sources by
oracle/ref/Makefile; the reference checkout is needed to regenerate).

Contents (all FP64, the reference's CPU Real):
  tet_*        48 seeded tets: rest shape Q, volume, compliances, gamma
               (ElementConstraint / Hydrostatic / Deviatoric ctors), C and
               grad C at a deformed state (both hydrostatic branches), three
               chained combined projections (CombinedNeohookeanConstraintProjector.cpp:98-179)
               and three chained scalar projections of each constraint
               (ConstraintProjector.hpp:111-172)
  col_*        32 seeded static collision constraints, three chained
               projections each, half of them separated (C > 0: no update)
  cube_*       unit cube of 4^3 hexes x 5 tets, E 3e3, nu 0.45, rho 1000,
               bottom fixed, rest + U(-1e-3, 1e-3) m, 10 sequential
               Gauss-Seidel sweeps, 50 substeps: final x and lambda
  block_*      6^3-hex block (0.1 m), per-tet E log-uniform [1e3, 1e5],
               nu 0.45, bottom fixed, 5 sweeps, 20 substeps: final x, lambda

Run: python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "oracle", "ref")]

OUT = os.path.join(HERE, "reference_kat.npz")
DT = 1e-3


def tet_cases(seed: int, n: int) -> dict:
    """Seeded tets: near-regular rest shapes at three scales, deformed by a
    random linear map (det above and below 1) plus noise, with random
    materials and vertex masses."""
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    X4, x4, E, nu, m4 = [], [], [], [], []
    for k in range(n):
        h = [1e-3, 1e-2, 0.1][k % 3]
        X = (base + rng.uniform(-0.2, 0.2, (4, 3))) * h
        A = np.eye(3) + rng.normal(0, 0.12, (3, 3))
        if k % 2:
            A *= 0.93  # J < 1: the Taylor branch of C_hyd
        else:
            A *= 1.06
        x = X @ A.T + rng.uniform(-0.02, 0.02, (4, 3)) * h
        X4.append(X)
        x4.append(x)
        E.append(float(np.exp(rng.uniform(np.log(1e3), np.log(1e5)))))
        nu.append(float(rng.uniform(0.3, 0.49)))
        m4.append(rng.uniform(0.5, 2.0, 4) * 1000.0 * h ** 3 / 24)
    return {"X4": np.array(X4), "x4": np.array(x4), "E": np.array(E), "nu": np.array(nu), "m4": np.array(m4)}


def col_cases(seed: int, n: int) -> dict:
    """Seeded static contacts: a face, vertex masses, barycentrics, a unit
    normal and a surface point placed so that C = n.(a - p) alternates sign."""
    rng = np.random.default_rng(seed)
    x3, m3, p, nrm, uvw = [], [], [], [], []
    for k in range(n):
        f = rng.uniform(-0.01, 0.01, (3, 3))
        b = rng.dirichlet([2, 2, 2])
        nn = rng.normal(size=3)
        nn /= np.linalg.norm(nn)
        a = b @ f
        depth = rng.uniform(1e-4, 2e-3) * (1 if k % 2 else -1)  # odd: separated (C > 0)
        p.append(a - depth * nn)
        x3.append(f)
        m3.append(rng.uniform(1e-6, 1e-4, 3))
        nrm.append(nn)
        uvw.append(b)
    return {"x3": np.array(x3), "m3": np.array(m3), "p": np.array(p), "n": np.array(nrm), "uvw": np.array(uvw)}


def tet_outputs(c: dict) -> dict:
    import refkat as R
    out = {k: [] for k in ["Q", "rest", "C", "gd", "gh", "comb_dx", "comb_lam", "dev_dx", "hyd_dx"]}
    for i in range(len(c["E"])):
        Q, r = R.rest(c["X4"][i], c["E"][i], c["nu"][i])
        C, gd, gh = R.evaluate(c["X4"][i], c["x4"][i], c["E"][i], c["nu"][i])
        dx, lam, _ = R.project_combined(c["X4"][i], c["x4"][i], c["m4"][i], c["E"][i], c["nu"][i], DT, 3)
        ddx, _ = R.project_single(0, c["X4"][i], c["x4"][i], c["m4"][i], c["E"][i], c["nu"][i], DT, 3)
        hdx, _ = R.project_single(1, c["X4"][i], c["x4"][i], c["m4"][i], c["E"][i], c["nu"][i], DT, 3)
        for k, v in zip(out, [Q, r, C, gd, gh, dx, lam, ddx, hdx]):
            out[k].append(v)
    return {k: np.array(v) for k, v in out.items()}


def col_outputs(c: dict) -> dict:
    import refkat as R
    dxs = []
    for i in range(len(c["m3"])):
        u, v, w = c["uvw"][i]
        dx, _ = R.project_collision(c["x3"][i], c["m3"][i], c["p"][i], c["n"][i], u, v, w, DT, 3)
        dxs.append(dx)
    return {"dx": np.array(dxs)}


def trajectories() -> dict:
    import oracle as O
    import refkat as R
    out = {}
    X, tets, _ = O.grid_mesh(4, 4, 4, 0.25)
    x0 = X + np.random.default_rng(7).uniform(-1e-3, 1e-3, X.shape)
    fixed = X[:, 2] == X[:, 2].min()
    x, lam = R.gs_steps(X, tets, 3e3, 0.45, 1000.0, fixed, DT, 9.81, 10, 50, x0=x0)
    out.update(cube_X=X, cube_tets=tets, cube_x0=x0, cube_x=x, cube_lam=lam)
    X, tets, _ = O.grid_mesh(6, 6, 6, 0.1 / 6)
    T = tets.shape[0]
    E = np.exp(np.random.default_rng(8).uniform(np.log(1e3), np.log(1e5), T))
    fixed = X[:, 2] == X[:, 2].min()
    x, lam = R.gs_steps(X, tets, E, 0.45, 1000.0, fixed, DT, 9.81, 5, 20)
    out.update(block_X=X, block_tets=tets, block_E=E, block_x=x, block_lam=lam)
    return out


def main():
    import refkat as R
    R.build()
    tc, cc = tet_cases(11, 48), col_cases(12, 32)
    to, co = tet_outputs(tc), col_outputs(cc)
    arrays = {f"tet_in_{k}": v for k, v in tc.items()}
    arrays.update({f"tet_out_{k}": v for k, v in to.items()})
    arrays.update({f"col_in_{k}": v for k, v in cc.items()})
    arrays.update({f"col_out_{k}": v for k, v in co.items()})
    arrays.update(trajectories())
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {len(arrays)} arrays")


if __name__ == "__main__":
    main()
