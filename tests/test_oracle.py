"""CPU tests of the oracle: pinned against the reference's own fixtures where
they exist, otherwise against known answers derived from the formulas."""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref_meshes(oracle_mod):
    return np.load(os.path.join(GOLDEN, "reference_meshes.npz"))


@pytest.mark.parametrize("n", [2, 4])
def test_grid_generator_reproduces_reference_cube_fixtures(ref_meshes, n):
    """resource/cube/cube{2,4}.msh were written by the reference's createBeamMsh."""
    X, tets, faces = O.grid_mesh(n, n, n, 1.0 / n, split=1)
    np.testing.assert_array_equal(X, ref_meshes[f"cube{n}_X"])
    np.testing.assert_array_equal(tets, ref_meshes[f"cube{n}_tets"])
    np.testing.assert_array_equal(faces, ref_meshes[f"cube{n}_faces"])


def test_msh_reader_single_tet(ref_meshes):
    X, T = ref_meshes["single_X"], ref_meshes["single_tets"]
    assert X.shape == (4, 3) and T.tolist() == [[0, 1, 2, 3]]
    Q, vol = np.zeros(9), np.zeros(1)
    import ctypes as C
    O.lib().xo_rest_shape(X.ctypes.data_as(C.c_void_p), Q.ctypes.data_as(C.c_void_p), vol.ctypes.data_as(C.c_void_p))
    D = (X[:3] - X[3]).T
    np.testing.assert_allclose(Q.reshape(3, 3).T, np.linalg.inv(D), rtol=1e-12, atol=1e-15)
    assert np.isclose(vol[0], abs(np.linalg.det(D)) / 6, rtol=1e-14)


@pytest.mark.parametrize("dims", [(2, 3, 4), (5, 2, 3), (4, 4, 4)])
def test_alternating_split_is_conforming(oracle_mod, dims):
    """Every interior triangle is shared by exactly two tets and the boundary
    triangles are exactly the generated surface faces."""
    X, tets, faces = O.grid_mesh(*dims, 0.1)
    from collections import Counter
    cnt = Counter()
    for t in tets:
        for tri in [(t[0], t[1], t[2]), (t[0], t[1], t[3]), (t[0], t[2], t[3]), (t[1], t[2], t[3])]:
            cnt[tuple(sorted(tri))] += 1
    assert max(cnt.values()) == 2
    assert {k for k, v in cnt.items() if v == 1} == {tuple(sorted(f)) for f in faces}
    # positive, equal-volume hexes
    D = np.stack([X[tets[:, i]] - X[tets[:, 3]] for i in range(3)], axis=2)
    vols = np.abs(np.linalg.det(D)) / 6
    np.testing.assert_allclose(vols.reshape(-1, 5).sum(1), 0.1 ** 3)


def _elem(x4, Q, gamma):
    import ctypes as C
    F = np.zeros(9); Cd = C.c_double(); Ch = C.c_double(); gd = np.zeros(12); gh = np.zeros(12)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    O.lib().xo_elem_eval(p(x4), p(Q), C.c_double(gamma), p(F), C.byref(Cd), C.byref(Ch), p(gd), p(gh))
    return F, Cd.value, Ch.value, gd, gh


@pytest.mark.parametrize("scale", [1.08, 0.93])  # J >= 1 (log branch) and J < 1 (Taylor branch)
def test_constraint_gradients_match_finite_differences(oracle_mod, scale):
    rng = np.random.default_rng(0)
    X4 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    D = (X4[:3] - X4[3]).T
    Q = np.linalg.inv(D).T.ravel()  # column-major storage of Q
    x4 = (X4 * scale + rng.normal(0, 0.01, X4.shape)).ravel()
    gamma = 0.3
    F, Cd, Ch, gd, gh = _elem(x4, Q, gamma)
    J = np.linalg.det(F.reshape(3, 3).T)
    assert (J >= 1) == (scale > 1)
    eps = 1e-7
    for i in range(12):
        xp, xm = x4.copy(), x4.copy()
        xp[i] += eps; xm[i] -= eps
        _, cdp, chp, _, _ = _elem(xp, Q, gamma)
        _, cdm, chm, _, _ = _elem(xm, Q, gamma)
        assert np.isclose(gd[i], (cdp - cdm) / (2 * eps), rtol=1e-5, atol=1e-7)
        assert np.isclose(gh[i], (chp - chm) / (2 * eps), rtol=1e-5, atol=1e-7)


def test_constraint_values_known_answers(oracle_mod):
    X4 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]])
    Q = np.linalg.inv((X4[:3] - X4[3]).T).T.ravel()
    F, Cd, Ch, _, _ = _elem(X4.ravel(), Q, 0.25)
    np.testing.assert_allclose(F.reshape(3, 3), np.eye(3), atol=1e-15)
    assert np.isclose(Cd, np.sqrt(3)) and np.isclose(Ch, -0.25)
    # uniform stretch s: C_d = sqrt(3) s, C_h = -gamma + log(s^3) for s >= 1
    s = 1.1
    _, Cd, Ch, _, _ = _elem((X4 * s).ravel(), Q, 0.25)
    assert np.isclose(Cd, np.sqrt(3) * s) and np.isclose(Ch, -0.25 + np.log(s ** 3))
    s = 0.9
    _, _, Ch, _, _ = _elem((X4 * s).ravel(), Q, 0.25)
    d = s ** 3 - 1
    assert np.isclose(Ch, -0.25 + d - d * d / 2 + d ** 3 / 3)


def test_lame_parameters_and_masses(oracle_mod):
    X, tets, faces = O.grid_mesh(2, 2, 2, 0.5)
    E, nu, rho = 2e4, 0.45, 1100.0
    o = O.Oracle(X, tets, faces, E, nu, rho)
    Q, vol, ad, ah, gm = o.tet_data()
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    np.testing.assert_allclose(ad, 1 / (mu * vol))
    np.testing.assert_allclose(ah, 1 / (lam * vol))
    np.testing.assert_allclose(gm, mu / lam)
    m = o.masses()
    assert np.isclose(m.sum(), rho * 1.0)  # unit cube
    ref = np.zeros(len(X))
    for t, v in zip(tets, vol):
        ref[t] += rho * v / 4
    np.testing.assert_allclose(m, ref)


@pytest.mark.parametrize("solver", [O.GAUSS_SEIDEL, O.JACOBI, O.COLOURED_GS])
def test_rest_state_is_stationary_without_gravity(oracle_mod, solver):
    """At F = I the deviatoric and hydrostatic forces cancel (gamma = mu/lambda)."""
    X, tets, faces = O.grid_mesh(3, 3, 3, 1 / 3)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, g=0.0, num_iter=10, solver=solver)
    o.time_steps(20)
    assert np.abs(o.positions() - X).max() < 1e-12


def test_free_fall_follows_discrete_update(oracle_mod):
    """Unconstrained fall: x_n = x_0 - g dt^2 n(n+1)/2 (XPBDMeshObject.cpp:462-468)."""
    X, tets, faces = O.grid_mesh(2, 2, 2, 0.5)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, num_iter=5, solver=O.GAUSS_SEIDEL)
    n = 40
    o.time_steps(n)
    dz = o.positions()[:, 2] - X[:, 2]
    np.testing.assert_allclose(dz, -9.81 * 1e-6 * n * (n + 1) / 2, rtol=1e-9)
    np.testing.assert_allclose(o.velocities()[:, 2], -9.81 * 1e-3 * n, rtol=1e-9)


def test_fixed_vertices_reset_and_residual_decreases(oracle_mod):
    X, tets, faces = O.grid_mesh(4, 4, 4, 0.25)
    o = O.Oracle(X, tets, faces, 5e4, 0.45, 1000.0, num_iter=8, solver=O.GAUSS_SEIDEL)
    fixed = X[:, 2] == 0
    o.set_fixed(fixed)
    o.time_steps(30, record=True)
    np.testing.assert_array_equal(o.positions()[fixed], X[fixed])
    h = o.res_history()
    assert h.shape == (9,) and h[-1] < h[0]


def test_jacobi_sums_updates_without_averaging(oracle_mod):
    """One Jacobi sweep equals x + the plain sum of per-tet updates
    (XPBDJacobiSolver.hpp:97-102), checked against per-tet projections."""
    import ctypes as C
    X, tets, faces = O.grid_mesh(2, 2, 2, 0.5)
    x0 = X + np.random.default_rng(7).uniform(-0.02, 0.02, X.shape)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, g=0.0, num_iter=1, solver=O.JACOBI)
    Q, vol, ad, ah, gm = o.tet_data()
    w = 1 / o.masses()
    acc = np.zeros_like(x0)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    for t in range(len(tets)):
        e = tets[t]
        x4 = np.ascontiguousarray(x0[e].ravel())
        lam = np.zeros(2); dx = np.zeros(12)
        at = np.array([ad[t] / 1e-6, ah[t] / 1e-6])
        O.lib().xo_project_combined(p(x4), p(np.ascontiguousarray(w[e])), p(np.ascontiguousarray(Q[t])), p(at),
                                    C.c_double(gm[t]), p(lam), p(dx))
        acc[e] += dx.reshape(4, 3)
    o.set_positions(x0)
    o.set_velocities(np.zeros_like(x0))
    o.update()
    np.testing.assert_allclose(o.positions(), x0 + acc, rtol=0, atol=1e-15)


def test_collision_cadence_uses_strict_accumulated_time(oracle_mod):
    """Detection runs when t - t_last > 1/rate on accumulated double time
    (Simulation.cpp:202,259-263)."""
    t, last, n = 0.0, 0.0, []
    for k in range(50):
        if t - last > 0.01:
            n.append(k)
            last = t
        t += 1e-3
    X, tets, faces = O.grid_mesh(2, 2, 2, 0.5)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, num_iter=1)
    o.set_collision_rate(100.0)
    o.set_spheres([[0.5, 0.5, -10.0]], [0.1])  # far away: detections find nothing
    o.time_steps(50)
    assert np.isclose(o.time, t)
    assert n[0] == 10 and n[1] - n[0] in (10, 11)


def test_oracle_matches_committed_golden_trajectories(oracle_mod):
    g = np.load(os.path.join(GOLDEN, "oracle_trajectories.npz"))
    X, tets, x0, fixed = g["X"], g["tets"], g["x0"], g["fixed"]
    faces = O.grid_mesh(3, 3, 3, 1 / 3)[2]
    for name, solver in [("gs", O.GAUSS_SEIDEL), ("jacobi", O.JACOBI), ("cgs", O.COLOURED_GS)]:
        o = O.Oracle(X, tets, faces, 4e3, 0.45, 1000.0, num_iter=5, solver=solver)
        o.set_positions(x0); o.set_fixed(fixed)
        o.time_steps(10, record=True)
        np.testing.assert_allclose(o.positions(), g[f"{name}_x"], rtol=0, atol=1e-13)
        np.testing.assert_allclose(o.lambdas(), g[f"{name}_lam"], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(o.res_history(), g[f"{name}_res"], rtol=1e-9)


def test_frank_wolfe_detection_finds_penetrating_faces(oracle_mod):
    X, tets, faces = O.grid_mesh(6, 6, 2, 1 / 6)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0)
    r = 0.2
    c = np.array([0.5, 0.5, X[:, 2].max() + r - 0.01])
    o.set_spheres(c, [r])
    n = o.detect()
    rows = o.contacts()
    assert n > 0
    for row in rows:
        f = int(row[1])
        u, v, w = row[2:5]
        assert np.isclose(u + v + w, 1) and min(u, v, w) > -1e-9
        p, nrm = row[5:8], row[8:11]
        assert np.isclose(np.linalg.norm(p - c), r)  # surface point on the sphere
        x = u * X[faces[f, 0]] + v * X[faces[f, 1]] + w * X[faces[f, 2]]
        assert np.linalg.norm(x - c) - r <= 1e-4  # penetrating (or within 1e-4)
        np.testing.assert_allclose(nrm, (x - c) / np.linalg.norm(x - c), atol=1e-9)


def test_greedy_colouring_is_valid_and_ordered(oracle_mod):
    X, tets, faces = O.grid_mesh(5, 4, 3, 0.1)
    n, col = O.greedy_colour(tets, len(X))
    assert 20 <= n <= 48
    for c in range(n):
        v = tets[col == c].ravel()
        assert len(np.unique(v)) == len(v)
    # greedy: each tet's colour is the smallest not used by earlier neighbours
    assert col[0] == 0


def test_first_order_free_body_translates_at_g_rho_dt_over_multiplier():
    """1st-order XPBD (FirstOrderXPBDMeshObject): with B = V_vertex * multiplier
    every vertex has m / B = rho / multiplier, so an unconstrained body at rest
    moves rigidly by -g rho dt / multiplier per step and stays undeformed
    (XPBDMeshObject.cpp:333-348, 449-456)."""
    import xpbd_gb300 as G
    X, tets, faces = G.grid_mesh(3, 3, 3, 0.1)
    for solver in (O.GAUSS_SEIDEL, O.JACOBI):
        o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, dt=1e-3, g=9.81, num_iter=5, solver=solver)
        o.set_first_order(5e4)
        o.time_steps(10)
        d = o.positions() - X
        assert np.abs(d[:, :2]).max() < 1e-12
        np.testing.assert_allclose(d[:, 2], -10 * 9.81 * 1000.0 * 1e-3 / 5e4, rtol=1e-9)
        o.close()


def test_first_order_damping_adjusted_to_material():
    """adjust-damping-to-material: B = V_vertex * multiplier * E_v / (1 + nu_v)."""
    import xpbd_gb300 as G
    X, tets, faces = G.grid_mesh(2, 2, 2, 0.1)
    o = O.Oracle(X, tets, faces, 2e3, 0.25, 1000.0, dt=1e-3, g=9.81, num_iter=3)
    o.set_first_order(10.0, adjust=True)
    o.time_steps(4)
    d = o.positions() - X
    np.testing.assert_allclose(d[:, 2], -4 * 9.81 * 1000.0 * 1e-3 / (10.0 * 2e3 / 1.25), rtol=1e-9)
    o.close()


def test_attachment_puts_its_vertex_on_the_target():
    """alpha = 0 and |grad C| = 1: one scalar projection moves the vertex by
    -(x - target); projected last in an iteration, it ends on the target."""
    import xpbd_gb300 as G
    X, tets, faces = G.grid_mesh(2, 2, 2, 0.1)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, dt=1e-3, g=0.0, num_iter=1)
    v = int(np.argmax(X[:, 2] + X[:, 0]))
    target = X[v] + np.array([0.01, -0.02, 0.03])
    o.add_attachment(v, target)
    o.update()
    np.testing.assert_allclose(o.positions()[v], target, atol=1e-12)
    o.close()
