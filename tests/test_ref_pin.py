"""The oracle pinned to the reference's own code.

tests/golden/reference_kat.npz holds inputs and outputs of the reference's
constraint and projector classes (ElementConstraint, Hydrostatic- and
DeviatoricConstraint, CombinedNeohookeanConstraintProjector.cpp:98-179,
ConstraintProjector.hpp:111-172, StaticDeformableCollisionConstraint.cpp:20-49),
compiled from the reference's sources by oracle/ref/Makefile and run by
tests/golden/make_ref_golden.py, plus two sequential Gauss-Seidel
trajectories driven through those projectors. The FP64 oracle
(oracle/xpbd_oracle.hpp) must reproduce them: per-element values to 1e-12 of
their scale, trajectories to 1e-10 of the mesh extent (bit-identical on the
machine that wrote them; the margin covers floating-point contraction on
other hosts). Where the reference library itself is built here
(oracle/_ref/libref_kat.so), fresh seeded cases are checked live as well.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden", "reference_kat.npz")
DT = 1e-3


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _close(a, b, rel=1e-12):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = max(np.abs(b).max(), 1e-300)
    assert np.abs(a - b).max() <= rel * scale, (np.abs(a - b).max(), scale)


def oracle_tet(X4, x4, m4, E, nu):
    """The oracle's per-element results for one tet, in the layout of the
    golden arrays."""
    tets = np.array([[0, 1, 2, 3]], np.int32)
    o = O.Oracle(np.ascontiguousarray(X4), tets, np.zeros((0, 3), np.int32), E, nu, 1000.0, dt=DT, num_iter=1, solver=O.GAUSS_SEIDEL)
    Q, vol, ad, ah, gm = o.tet_data()
    o.close()
    Q, gamma = np.ascontiguousarray(Q[0]), float(gm[0])
    L = O.lib()
    F = np.zeros(9); Cd = C.c_double(); Ch = C.c_double(); gd = np.zeros(12); gh = np.zeros(12)
    x = np.ascontiguousarray(x4, np.float64).reshape(-1).copy()
    L.xo_elem_eval(_p(x), _p(Q), C.c_double(gamma), _p(F), C.byref(Cd), C.byref(Ch), _p(gd), _p(gh))
    w = np.ascontiguousarray(1.0 / np.asarray(m4, float))
    at = np.array([ad[0] / DT ** 2, ah[0] / DT ** 2])
    lam = np.zeros(2)
    comb_dx, comb_lam = [], []
    for _ in range(3):
        dx = np.zeros(12)
        L.xo_project_combined(_p(x), _p(w), _p(Q), _p(at), C.c_double(gamma), _p(lam), _p(dx))
        x += dx
        comb_dx.append(dx)
        comb_lam.append(lam.copy())
    single = []
    for which in (0, 1):
        x = np.ascontiguousarray(x4, np.float64).reshape(-1).copy()
        lam1 = np.zeros(1)
        rows = []
        for _ in range(3):
            dx = np.zeros(12)
            L.xo_project_single(which, _p(x), _p(w), _p(Q), C.c_double(at[which]), C.c_double(gamma), _p(lam1), _p(dx))
            x += dx
            rows.append(dx)
        single.append(np.array(rows))
    return {"Q": Q, "rest": np.array([vol[0], ad[0], ah[0], gamma]), "C": np.array([Cd.value, Ch.value]), "gd": gd,
            "gh": gh, "comb_dx": np.array(comb_dx), "comb_lam": np.array(comb_lam), "dev_dx": single[0],
            "hyd_dx": single[1]}


def oracle_contact(x3, m3, p, n, uvw):
    L = O.lib()
    x = np.ascontiguousarray(x3, np.float64).reshape(-1).copy()
    w = np.ascontiguousarray(1.0 / np.asarray(m3, float))
    lam = np.zeros(1)
    rows = []
    for _ in range(3):
        dx = np.zeros(9)
        L.xo_project_contact(_p(x), _p(w), C.c_double(uvw[0]), C.c_double(uvw[1]), C.c_double(uvw[2]),
                             _p(np.ascontiguousarray(p, float)), _p(np.ascontiguousarray(n, float)), _p(lam), _p(dx))
        x += dx
        rows.append(dx)
    return np.array(rows)


def _check_tets(cases, outs, n=None):
    n = len(cases["E"]) if n is None else n
    for i in range(n):
        got = oracle_tet(cases["X4"][i], cases["x4"][i], cases["m4"][i], cases["E"][i], cases["nu"][i])
        for k in ["Q", "rest", "C", "gd", "gh", "comb_dx", "comb_lam", "dev_dx", "hyd_dx"]:
            _close(got[k], outs[k][i])


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def test_golden_vectors_cover_both_hydrostatic_branches_and_both_contact_states(gold):
    X4, x4 = gold["tet_in_X4"], gold["tet_in_x4"]
    J = [np.linalg.det((x[:3] - x[3]).T) / np.linalg.det((X[:3] - X[3]).T) for X, x in zip(X4, x4)]
    assert min(J) < 1 < max(J)
    dx = gold["col_out_dx"]
    assert (np.abs(dx).reshape(len(dx), -1).max(1) == 0).any() and (np.abs(dx).reshape(len(dx), -1).max(1) > 0).any()


def test_oracle_elements_match_reference_vectors(oracle_mod, gold):
    cases = {k[len("tet_in_"):]: v for k, v in gold.items() if k.startswith("tet_in_")}
    outs = {k[len("tet_out_"):]: v for k, v in gold.items() if k.startswith("tet_out_")}
    _check_tets(cases, outs)


def test_oracle_contacts_match_reference_vectors(oracle_mod, gold):
    for i in range(len(gold["col_in_m3"])):
        got = oracle_contact(gold["col_in_x3"][i], gold["col_in_m3"][i], gold["col_in_p"][i], gold["col_in_n"][i],
                             gold["col_in_uvw"][i])
        ref = gold["col_out_dx"][i]
        assert np.abs(got - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-9)


@pytest.mark.parametrize("name,iters,steps", [("cube", 10, 50), ("block", 5, 20)])
def test_oracle_sequential_gauss_seidel_matches_reference_trajectory(oracle_mod, gold, name, iters, steps):
    X, tets = gold[f"{name}_X"], gold[f"{name}_tets"]
    T = tets.shape[0]
    E = gold[f"{name}_E"] if f"{name}_E" in gold else np.full(T, 3e3)
    o = O.Oracle(X, tets, np.zeros((0, 3), np.int32), E, 0.45, 1000.0, dt=DT, g=9.81, num_iter=iters, solver=O.GAUSS_SEIDEL)
    if f"{name}_x0" in gold:
        o.set_positions(gold[f"{name}_x0"])
    o.set_fixed(X[:, 2] == X[:, 2].min())
    o.time_steps(steps)
    extent = float((X.max(0) - X.min(0)).max())
    err = np.abs(o.positions() - gold[f"{name}_x"]).max()
    assert np.abs(gold[f"{name}_x"] - X).max() > 1e-4 * extent  # the reference run deformed
    assert err <= 1e-10 * extent, err
    _close(o.lambdas(), gold[f"{name}_lam"], rel=1e-8)
    o.close()


def _refkat():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import refkat
    if not os.path.exists(refkat.LIB):
        if not refkat.available():
            pytest.skip("the reference checkout is not on this machine; the committed vectors cover it")
        refkat.build()
    return refkat


def test_live_reference_elements_match_oracle_on_fresh_cases(oracle_mod):
    """New seeds through the reference library itself, when it is built here."""
    _refkat()
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_ref_golden as M
    cases = M.tet_cases(1234, 24)
    _check_tets(cases, M.tet_outputs(cases))
    cc = M.col_cases(4321, 16)
    co = M.col_outputs(cc)
    for i in range(len(cc["m3"])):
        got = oracle_contact(cc["x3"][i], cc["m3"][i], cc["p"][i], cc["n"][i], cc["uvw"][i])
        assert np.abs(got - co["dx"][i]).max() <= 1e-12 * max(np.abs(co["dx"][i]).max(), 1e-9)
