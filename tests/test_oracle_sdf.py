"""CPU checks of the oracle's SDF primitives (BoxSDF, CylinderSDF,
SphereSDF in src/geometry/): known distances and gradients, rotations by
quaternion, and finite differences away from edges."""
import numpy as np
import pytest

import oracle as O

ID = [0, 0, 0, 1]


def _to_body(p, q, x):
    u, w = np.asarray(q[:3]) / np.dot(q, q), q[3] / np.dot(q, q)
    u = -u
    v = np.asarray(x) - p
    return 2 * np.dot(u, v) * u + (2 * w * w - 1) * v + 2 * w * np.cross(u, v)


@pytest.mark.parametrize("kind,dims,x,expect", [
    (O.PRIM_BOX, [2, 2, 2], [3, 0, 0], [2, 1, 0, 0]),
    (O.PRIM_BOX, [2, 2, 2], [0.5, 0, 0], [-0.5, 1, 0, 0]),
    (O.PRIM_BOX, [2, 2, 2], [2, 2, 0], [np.sqrt(2), np.sqrt(0.5), np.sqrt(0.5), 0]),
    (O.PRIM_BOX, [2, 4, 6], [0, -1.5, 0], [-0.5, 0, -1, 0]),
    (O.PRIM_CYLINDER, [1, 2, 0], [3, 0, 0], [2, 1, 0, 0]),
    (O.PRIM_CYLINDER, [1, 2, 0], [0, 0, 3], [2, 0, 0, 1]),
    (O.PRIM_CYLINDER, [1, 2, 0], [0.2, 0, 0.1], [-0.8, 1, 0, 0]),
    (O.PRIM_CYLINDER, [1, 2, 0], [0, 0.1, -0.95], [-0.05, 0, 0, -1]),
    (O.PRIM_SPHERE, [0.5, 0, 0], [0, 2, 0], [1.5, 0, 1, 0]),
])
def test_known_values(kind, dims, x, expect):
    np.testing.assert_allclose(O.prim_eval(kind, [0, 0, 0], ID, dims, x), expect, atol=1e-12)


def test_rotation_and_translation():
    # box 2 x 4 x 2 turned 90 degrees about z, centred at (1, 0, 0)
    s = np.sin(np.pi / 4)
    q = [0, 0, s, np.cos(np.pi / 4)]
    r = O.prim_eval(O.PRIM_BOX, [1, 0, 0], q, [2, 4, 2], [4, 0, 0])
    # body frame: the point is 3 along -y, the face is 2 away: distance 1, normal +x in the world
    np.testing.assert_allclose(r, [1, 1, 0, 0], atol=1e-12)


@pytest.mark.parametrize("kind,dims", [(O.PRIM_BOX, [0.3, 0.5, 0.7]), (O.PRIM_CYLINDER, [0.25, 0.8, 0])])
def test_gradient_matches_central_differences(kind, dims):
    rng = np.random.default_rng(kind)
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    p = rng.uniform(-0.2, 0.2, 3)
    checked = 0
    for _ in range(400):
        x = p + rng.uniform(-1.0, 1.0, 3)
        v = O.prim_eval(kind, p, q, dims, x)
        if abs(v[0]) < 0.05:
            continue
        if kind == O.PRIM_CYLINDER:
            # at the rim (outside both radially and axially) the reference's
            # gradient is the normalised body-frame position, not the
            # distance's gradient: skip those points
            b = _to_body(p, q, x)
            if np.hypot(b[0], b[1]) > dims[0] and abs(b[2]) > dims[1] / 2:
                continue
        h = 1e-6
        fd = [(O.prim_eval(kind, p, q, dims, x + h * e)[0] - O.prim_eval(kind, p, q, dims, x - h * e)[0]) / (2 * h)
              for e in np.eye(3)]
        if v[0] > 0:  # outside: the gradient is the distance's gradient
            np.testing.assert_allclose(v[1:], fd, atol=1e-5)
            checked += 1
        else:  # inside: unit normal of the nearest face (box) or side / cap (cylinder)
            assert abs(np.linalg.norm(v[1:]) - 1) < 1e-9
            np.testing.assert_allclose(v[1:], fd, atol=1e-5)
            checked += 1
    assert checked > 100
