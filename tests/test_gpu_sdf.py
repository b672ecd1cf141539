"""Box and cylinder SDFs (BoxSDF, CylinderSDF) on the GPU: values and
gradients against the FP32 oracle, collision detection against the oracle,
and a Gauss-Seidel trajectory with box contacts against the FP64 oracle."""
import numpy as np
import pytest

import oracle as O
import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _quat(seed):
    q = np.random.default_rng(seed).standard_normal(4)
    return q / np.linalg.norm(q)


@pytest.mark.parametrize("kind,dims", [(G.SDF_SPHERE, [0.3, 0, 0]), (G.SDF_BOX, [0.3, 0.5, 0.7]),
                                       (G.SDF_CYLINDER, [0.25, 0.8, 0])])
def test_sdf_values_and_gradients_match_fp32_oracle(lib, kind, dims):
    rng = np.random.default_rng(kind)
    q, p = _quat(kind + 10), rng.uniform(-0.2, 0.2, 3)
    pts = p + rng.uniform(-1.0, 1.0, (500, 3))
    got = G.sdf_eval(kind, p, q, dims, pts)
    ref = np.array([O.prim_eval(kind, p, q, dims, x, precision=32) for x in pts])
    np.testing.assert_allclose(got[:, 0], ref[:, 0], atol=2e-6)
    np.testing.assert_allclose(got[:, 1:], ref[:, 1:], atol=2e-5)


def _beam():
    w = W.beam(nl=20, nw=4, nh=4, length=0.1)
    x = w.X.copy()
    x[:, 2] -= 0.5e-3 * np.sin(np.pi * x[:, 1] / x[:, 1].max())
    return w, x


# the beam is 0.02 wide (x), 0.1 long (y), 0.02 high (z): both primitives
# press 1.5 mm into its top face around mid-length
PRIMS = {
    "box": (G.SDF_BOX, [0.01, 0.05, 0.02 - 0.0015 + 0.01], [0.04, 0.03, 0.02]),
    "cylinder": (G.SDF_CYLINDER, [0.01, 0.05, 0.02 - 0.0015 + 0.015], [0.02, 0.03, 0.0]),
}


@pytest.mark.parametrize("name", ["box", "cylinder"])
def test_detection_matches_fp32_oracle(lib, name):
    kind, pos, dims = PRIMS[name]
    q = np.array([0, 0, np.sin(0.2), np.cos(0.2)])  # turned 23 degrees about z
    w, x = _beam()
    s = G.XPBDSolver(w.X, w.tets, w.faces, w.E, w.nu, w.rho, num_iters=1)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, precision=32)
    s.set_positions(x); o.set_positions(x)
    s.set_sdfs([kind], [pos], [q], [dims]); o.set_prims([kind], [pos], [q], [dims])
    s.detect_collisions()
    nref = o.detect()
    assert nref > 0
    fg = {int(r[1]): r for r in s.collisions()}
    fo = {int(r[1]): r for r in o.contacts()}
    assert len(set(fg) ^ set(fo)) <= max(1, nref // 50)
    for f in set(fg) & set(fo):
        np.testing.assert_allclose(fg[f][2:11], fo[f][2:11], atol=5e-5)
    s.close()
    o.close()


def test_box_contacts_trajectory_matches_fp64_oracle(lib):
    """A fixed box pressed 1.5 mm into the beam's top: 40 Gauss-Seidel steps with
    the GPU's contacts fed to the FP64 oracle at every detection."""
    kind, pos, dims = PRIMS["box"]
    q = np.array([0, 0, 0, 1.0])
    w = W.beam(nl=20, nw=4, nh=4, length=0.1)
    s = G.XPBDSolver(w.X, w.tets, w.faces, w.E, w.nu, w.rho, num_iters=8)
    s.fix_vertices(w.fixed)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, num_iter=8, solver=O.COLOURED_GS)
    o.set_order(s.sweep_order())
    o.set_fixed(w.fixed)
    s.set_sdfs([kind], [pos], [q], [dims])
    t, last, interval = 0.0, 0.0, 1.0 / w.collision_rate
    n = 0
    for k in range(40):
        if t - last > interval:
            s.detect_collisions()
            rows = s.collisions()
            n += len(rows)
            o.set_contacts(rows)
        s.update(); s.velocity_update()
        o.update(); o.velocity_update()
        if t - last > interval:
            last = t
        t += w.dt
    assert n > 0
    err = np.abs(s.positions() - o.positions()).max()
    assert err <= 1e-4 * 0.1, err
    s.close()
    o.close()
