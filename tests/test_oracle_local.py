"""CPU checks of the oracle's local collision iterations
(XPBDMeshObject.cpp:472-505, 764-825): the gathered tet list keeps the
reference's duplicates and order, and extra local passes lower the residual
while the contacts stay satisfied."""
import numpy as np

import oracle as O


def _beam(solver=O.GAUSS_SEIDEL, local=0):
    X, tets, faces = O.grid_mesh(4, 20, 4, 0.005)
    T = tets.shape[0]
    o = O.Oracle(X, tets, faces, np.full(T, 1e4), np.full(T, 0.49), np.full(T, 1000.0), num_iter=5, solver=solver)
    o.set_fixed(X[:, 1] == X[:, 1].min())
    c = np.array([[X[:, 0].max() / 2, X[:, 1].max() / 2, X[:, 2].max() + 0.02 - 0.002]])
    o.set_spheres(c, [0.02])
    if local:
        o.set_local_iterations(local)
    return X, tets, faces, o


def test_local_passes_lower_the_residual_and_keep_contacts():
    """Contacts (alpha = 0, projected last in each pass) stay satisfied; the
    extra passes over the tets around them lower the constraint residual."""
    res = {}
    for local in (0, 1, 4):
        X, tets, faces, o = _beam(local=local)
        o.detect()
        assert len(o.contacts()) > 0
        o.update()
        res[local] = o.residual_norm()
        x = o.positions()
        for r in o.contacts():
            f = faces[int(r[1])]
            q = r[2] * x[f[0]] + r[3] * x[f[1]] + r[4] * x[f[2]]
            assert np.dot(r[8:11], q - r[5:8]) >= -1e-12
        o.close()
    assert res[4] < res[1] < res[0], res


def test_zero_local_passes_change_nothing():
    a = _beam()[3]
    b = _beam(local=0)[3]
    b.set_local_iterations(0)
    for o in (a, b):
        o.detect()
        o.update()
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_gathered_list_matches_the_reference_rule():
    """After the global solve, the reference lists, for each contact with
    lambda != 0 and each of its vertices, every attached element in ascending
    order, duplicates kept."""
    X, tets, faces, o = _beam()
    o.detect()
    o.update()
    lam = o.contacts()[:, 11]
    assert (lam != 0).any()
    attached = [[] for _ in range(X.shape[0])]
    for t, e in enumerate(tets):
        for v in e:
            attached[v].append(t)
    expect = [t for r in o.contacts() if r[11] != 0 for v in faces[int(r[1])] for t in attached[v]]
    assert len(expect) > len(set(expect))  # duplicates are part of the rule
    np.testing.assert_array_equal(o.local_tets(), expect)
    o.close()
