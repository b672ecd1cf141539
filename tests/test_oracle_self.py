"""Self-collisions in the oracle (self-collisions: true) against numpy
restatements of the reference:
  selfCollisionCheck                          src/simobject/XPBDMeshObject.cpp:719-762
  EmbreeScene::tetMeshSelfCollisionQuery      src/geometry/embree/EmbreeScene.cpp:369-393
  isPointInTetrahedron                        src/geometry/embree/EmbreeTetMeshGeometry.cpp:20-47
  closestSurfaceFaceToPointInTet              src/geometry/DeformableMeshSDF.cpp:68-82
  DeformableDeformableCollisionConstraint     src/solver/constraint/DeformableDeformableCollisionConstraint.cpp
"""
import numpy as np
import pytest

import oracle as O
import xpbd_gb300 as G


def two_cubes(n=3, gap=0.005, shift=(0.0, 0.01, 0.005)):
    """Two n^3-hex cubes of 0.1 m in one mesh, side by side along x."""
    Xa, ta, fa = G.grid_mesh(n, n, n, 0.1 / n)
    Xb = Xa + np.array([0.1 + gap, shift[1], shift[2]])
    return np.vstack([Xa, Xb]), np.vstack([ta, ta + len(Xa)]), np.vstack([fa, fa + len(Xa)]), len(Xa)


def skew(v):
    return np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])


def contact_eval(q, p1, p2, p3):
    """C and gradient exactly as the reference writes them (matrix form)."""
    a = np.cross(p2 - p1, p3 - p1)
    an = np.linalg.norm(a)
    C = (q - p1).dot(a) / an + 1e-5
    M = np.eye(3) / an - np.outer(a, a) / an ** 3
    gq = a / an
    gp1 = -a / an + (q - p1) @ M @ skew(p3 - p2)
    gp2 = (q - p1) @ M @ skew(p1 - p3)
    gp3 = (q - p2) @ M @ skew(p2 - p1)
    return C, np.concatenate([gq, gp1, gp2, gp3])


def test_constraint_value_and_gradient_known_answers():
    X, tets, faces, na = two_cubes()
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, g=0.0)
    rng = np.random.default_rng(5)
    x = X + rng.uniform(-0.01, 0.01, X.shape)
    o.set_positions(x)
    for f in (0, 7, 31, len(faces) - 1):
        v = int(rng.integers(0, len(X)))
        C, g = o.self_contact_eval(v, f)
        Ce, ge = contact_eval(x[v], *x[faces[f]])
        assert abs(C - Ce) <= 1e-13
        np.testing.assert_allclose(g, ge, rtol=0, atol=1e-12)
    o.close()


def in_tet_f(p, v0, v1, v2, v3):
    f = np.float32

    def same(p, a, b, c, d):
        ab, ac = (b - a).astype(f), (c - a).astype(f)
        n = np.array([ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]],
                     dtype=f)
        sp = f(f(f(n[0] * f(p[0] - a[0])) + f(n[1] * f(p[1] - a[1]))) + f(n[2] * f(p[2] - a[2])))
        sd = f(f(f(n[0] * f(d[0] - a[0])) + f(n[1] * f(d[1] - a[1]))) + f(n[2] * f(d[2] - a[2])))
        return f(sp * sd) >= 0
    return same(p, v0, v1, v2, v3) and same(p, v0, v1, v3, v2) and same(p, v0, v2, v3, v1) and same(p, v1, v2, v3, v0)


def tri_dist(p, a, b, c):
    """Distance to a triangle by projecting onto its plane and, when outside,
    onto its edges (float64; used for the ranking only)."""
    n = np.cross(b - a, c - a)
    n = n / np.linalg.norm(n)
    q = p - n.dot(p - a) * n
    def inside(q):
        return all(np.cross(y - x, q - x).dot(n) >= 0 for x, y in ((a, b), (b, c), (c, a)))
    if inside(q):
        return np.linalg.norm(p - q)
    best = np.inf
    for x, y in ((a, b), (b, c), (c, a)):
        t = np.clip((p - x).dot(y - x) / (y - x).dot(y - x), 0, 1)
        best = min(best, np.linalg.norm(p - (x + t * (y - x))))
    return best


def expected_self_contacts(x, X, tets, faces):
    surf = np.unique(faces)
    xf, Xf = x.astype(np.float32), X.astype(np.float32)
    out = []
    for v in surf:
        hit = -1
        for t, e in enumerate(tets):
            if v in e:
                continue
            if in_tet_f(xf[v], *xf[e]):
                hit = t
                break
        if hit < 0:
            continue
        e = tets[hit]
        Dm = np.column_stack([X[e[i]] - X[e[3]] for i in range(3)])
        Ds = np.column_stack([x[e[i]] - x[e[3]] for i in range(3)])
        F = Ds @ np.linalg.inv(Dm)
        if abs(np.linalg.det(F)) < 1e-8:
            continue
        Xm = (np.linalg.inv(F) @ (x[v] - x[e[3]]) + X[e[3]]).astype(np.float32).astype(float)
        d = [tri_dist(Xm, *Xf[fc].astype(float)) for fc in faces]
        out.append((v, int(np.argmin(d))))
    return out


def test_detection_finds_surface_vertices_inside_other_tets():
    """The first cube pushed 6 mm into the second: each of its penetrating
    surface vertices pairs with the closest face of the second cube's rest
    surface, in vertex order (a numpy restatement of the query chain)."""
    X, tets, faces, na = two_cubes(gap=0.002, shift=(0, 0.013, 0.007))
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, g=0.0)
    o.enable_self_collisions()
    x = X.copy()
    x[:na, 0] += 0.008
    o.set_positions(x)
    o.detect()
    got = [(int(r[0]), int(r[1])) for r in o.self_contacts()]
    exp = expected_self_contacts(x, X, tets, faces)
    assert len(got) >= 4
    assert got == exp
    o.close()


@pytest.mark.parametrize("solver", [O.GAUSS_SEIDEL, O.JACOBI])
def test_colliding_cubes_stop_each_other(solver):
    """Two cubes of one mesh moving at 1 m/s toward each other: without
    self-collisions they pass through, with them they are stopped within
    about a hex width."""
    X, tets, faces, na = two_cubes()
    ends = {}
    for on in (False, True):
        o = O.Oracle(X, tets, faces, 2e4, 0.45, 1000.0, g=0.0, num_iter=8, solver=solver)
        o.set_collision_rate(1000.0)
        if on:
            o.enable_self_collisions()
        v = np.zeros_like(X)
        v[:na, 0], v[na:, 0] = 1.0, -1.0
        o.set_velocities(v)
        o.time_steps(20)
        x = o.positions()
        ends[on] = x[:na, 0].max() - x[na:, 0].min()
        o.close()
    assert ends[False] > 0.03                 # 4 cm of overlap
    assert 0 < ends[True] < 0.1 / 3 * 0.5     # stopped inside half a hex
