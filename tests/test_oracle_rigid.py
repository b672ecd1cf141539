"""Free rigid bodies in the oracle (RigidObject with fixed: false and the
two-way RigidDeformableCollisionConstraint), checked against independent
numpy restatements of the reference's formulas:
  RigidObject::update / velocityUpdate      src/simobject/RigidObject.cpp:41-77
  RigidDeformableCollisionConstraint        src/solver/constraint/RigidDeformableCollisionConstraint.cpp:35-55
  RigidBodyConstraintProjector::project     include/solver/xpbd_projector/RigidBodyConstraintProjector.hpp:97-158
  PositionalRigidBodyXPBDHelper::update     include/solver/constraint/RigidBodyConstraint.hpp
"""
import numpy as np
import pytest

import oracle as O
import xpbd_gb300 as G


def qmul(a, b):
    return np.array([a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1],
                     a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2],
                     a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0],
                     a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2]])


def qrot(v, q):
    u = q[:3]
    return 2 * u.dot(v) * u + (2 * q[3] ** 2 - 1) * v + 2 * q[3] * np.cross(u, v)


def qinv(q):
    return np.array([-q[0], -q[1], -q[2], q[3]]) / q.dot(q)


def _sphere_scene(g=0.0, solver=O.GAUSS_SEIDEL, c=(0.05, 0.05, 0.148), r=0.05, v=(0, 0, 0), w=(0, 0, 0)):
    X, tets, faces = G.grid_mesh(1, 1, 1, 0.1)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, dt=1e-3, g=g, num_iter=1, solver=solver)
    c = np.asarray(c, float)
    q = np.array([0.0, 0.0, 0.0, 1.0])
    o.set_prims([0], [c], [q], [[r, 0, 0]])
    m = 4.0 / 3.0 * 3.1415 * r ** 3 * 500.0
    inertia = np.full(3, 2.0 / 5.0 * m * r * r)
    o.set_rigid_body(0, c, q, m, inertia, v, w)
    return o, X, m, inertia


def test_free_fall_is_semi_implicit_euler():
    """No contact: v_n = v0 - n g dt e_z, p_n = p0 + dt sum v_k, and the
    velocity update returns v_n."""
    p0, v0 = np.array([0.3, 0.2, 1.0]), np.array([0.1, -0.2, 0.4])
    o, _, _, _ = _sphere_scene(g=9.81, c=p0, r=0.05, v=v0)
    n, dt, g = 37, 1e-3, 9.81
    o.time_steps(n)
    p, q, v, w = o.rigid_body(0)
    vn = v0 - n * g * dt * np.array([0, 0, 1.0])
    pn = p0 + n * dt * v0 - g * dt * dt * n * (n + 1) / 2 * np.array([0, 0, 1.0])
    # (p - p_prev) / dt loses ~1e-16 / dt to cancellation
    np.testing.assert_allclose(v, vn, rtol=0, atol=1e-11)
    np.testing.assert_allclose(p, pn, rtol=0, atol=1e-12)
    np.testing.assert_allclose(q, [0, 0, 0, 1], atol=1e-15)
    o.close()


def test_torque_free_spin_follows_the_quaternion_recurrence():
    """A box spinning about a principal axis: the body-frame Euler step adds
    nothing (w x Iw = 0), q <- normalise(q + dt/2 [w, 0] q), and the velocity
    update reads w back from q q_prev^-1."""
    X, tets, faces = G.grid_mesh(1, 1, 1, 0.1)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, dt=1e-3, g=0.0, num_iter=1)
    c, q0 = np.array([2.0, 0, 0]), np.array([0.0, 0.0, 0.0, 1.0])
    size = np.array([0.1, 0.2, 0.3])
    o.set_prims([1], [c], [q0], [size])
    m = size.prod() * 800.0
    inertia = m / 12 * np.array([size[1] ** 2 + size[2] ** 2, size[0] ** 2 + size[2] ** 2, size[0] ** 2 + size[1] ** 2])
    w0 = np.array([0.0, 0.0, 3.0])
    o.set_rigid_body(0, c, q0, m, inertia, (0, 0, 0), w0)
    q, w, dt = q0.copy(), w0.copy(), 1e-3
    for _ in range(25):
        q_prev = q.copy()
        q = q + 0.5 * dt * qmul(np.append(w, 0.0), q)
        q = q / np.linalg.norm(q)
        dq = qmul(q, qinv(q_prev))
        w = 2 / dt * dq[:3] * (-1 if dq[3] < 0 else 1)
    o.time_steps(25)
    p, qo, v, wo = o.rigid_body(0)
    np.testing.assert_allclose(qo, q, atol=1e-13)
    np.testing.assert_allclose(wo, w, atol=1e-10)
    np.testing.assert_allclose(p, c, atol=1e-15)
    o.close()


def _expected_contacts(o, X, m, inertia, c, r, jacobi):
    """One sweep of the rigid contacts from positions X and the body at c
    (identity orientation), restated from the reference's formulas."""
    x = X.astype(float).copy()
    w_inv = 1.0 / o.masses()
    p, q = np.array(c, float), np.array([0, 0, 0, 1.0])
    acc_x, acc_p, acc_q = np.zeros_like(x), np.zeros(3), np.zeros(4)
    for row in o.contacts():
        f = int(row[1])
        vs = o.faces[f]
        b, pt, n = row[2:5], row[5:8], row[8:11]
        a = sum(b[i] * x[vs[i]] for i in range(3))
        C = np.linalg.norm(a - p) - r          # SphereSDF at the current pose
        if C > 0:
            continue
        L = sum(w_inv[vs[i]] * np.dot(b[i] * n, b[i] * n) for i in range(3))
        dl = -C / L
        dx = [w_inv[vs[i]] * (b[i] * n) * dl for i in range(3)]
        d = -n
        rb = qrot(pt - p, qinv(q))
        nb = qrot(d, qinv(q))
        dp = dl * d / m
        wb = 0.5 * (1.0 / inertia) * np.cross(rb, dl * nb)
        dq = qmul(np.append(qrot(wb, q), 0.0), q)
        if jacobi:
            for i in range(3):
                acc_x[vs[i]] += dx[i]
            acc_p += dp
            acc_q += dq
        else:
            for i in range(3):
                x[vs[i]] += dx[i]
            p, q = p + dp, q + dq
    if jacobi:
        x, p, q = x + acc_x, p + acc_p, q + acc_q
    return x, p, q


@pytest.mark.parametrize("solver", [O.GAUSS_SEIDEL, O.JACOBI])
def test_rigid_contacts_known_answer(solver):
    """A free sphere 2 mm into the top of a resting 1-hex cube, no gravity, one
    iteration: the rest state leaves the elastic pass idle, so the vertices
    and the body move exactly by the rigid contact projections (Gauss-Seidel:
    each from the previous one's result; Jacobi: all from one state, summed)."""
    c, r = (0.05, 0.05, 0.148), 0.05
    o, X, m, inertia = _sphere_scene(solver=solver, c=c, r=r)
    o.detect()
    ct = o.contacts()
    assert len(ct) >= 2
    x_exp, p_exp, q_exp = _expected_contacts(o, X, m, inertia, c, r, solver == O.JACOBI)
    o.update()
    p, q, _, _ = o.rigid_body(0)
    np.testing.assert_allclose(o.positions(), x_exp, atol=1e-12)
    np.testing.assert_allclose(p, p_exp, atol=1e-14)
    np.testing.assert_allclose(q, q_exp, atol=1e-12)
    # the contact pushes the sphere up and the top face down
    assert p[2] > c[2] and o.positions()[X[:, 2] == X[:, 2].max(), 2].min() < X[:, 2].max()
    o.close()


@pytest.mark.parametrize("solver", [O.GAUSS_SEIDEL, O.JACOBI])
def test_contact_impulses_balance(solver):
    """Each rigid contact gives the face sum(m_i dx_i) = n dlam and the body
    m dp = -n dlam, and the elastic projections are internal: without gravity
    the mass-weighted displacement of vertices plus body stays zero over a
    whole update of several iterations."""
    c, r = (0.05, 0.05, 0.146), 0.05
    o, X, m, inertia = _sphere_scene(solver=solver, c=c, r=r)
    o.set_num_iter(6)
    o.detect()
    o.update()
    p, _, _, _ = o.rigid_body(0)
    total = (o.masses()[:, None] * (o.positions() - X)).sum(0) + m * (p - np.asarray(c))
    assert np.abs(p - np.asarray(c)).max() > 1e-6
    np.testing.assert_allclose(total, 0.0, atol=1e-15)
    o.close()
