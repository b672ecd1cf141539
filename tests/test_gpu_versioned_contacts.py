"""Static contacts inside the versioned sweep (gs_variant 4 with surface
faces): every iteration's contact phases run in the same cooperative launch
as the patch colours, ordered by vertex versions that count, per vertex and
iteration, its patches and then its faces with an active contact (face-colour
order). The projections and their order are those of the colour launches
(XPBDGaussSeidelSolver.hpp:29-80, contacts after the tets in projector type
order, XPBDTypedefs.hpp:55-56), so the trajectories agree with them within
FP32 rounding drift, reruns are bit-identical, and a batch equals its
instances stepped alone."""
import numpy as np
import pytest

import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _beam():
    w = W.beam(nl=20, nw=4, nh=4, length=0.1)
    w.sphere_r = 0.02
    w.sphere_c0 = np.array([w.X[:, 0].max() / 2, w.X[:, 1].max() / 2, w.X[:, 2].max() + 0.02 - 0.002])
    return w


def _run(w, var, steps, **kw):
    s = W.make_solver(w, num_iters=8, gs_variant=var, **kw)
    per_step = []
    ncontacts = 0
    for k in range(steps):
        l0 = s.launch_count()
        W.drive_gpu(s, w, k + 1)
        s.step(1)
        per_step.append(s.launch_count() - l0)
        ncontacts += len(s.collisions())
    s.synchronize()
    out = (s.positions(), ncontacts, per_step, s.health())
    s.close()
    return out


def test_versioned_sweep_with_contacts_matches_colour_launches(lib):
    w = _beam()
    a = _run(w, 4, 40)
    b = _run(w, 4, 40)
    ref = _run(w, 0, 40)
    assert a[1] > 0                           # contacts were active
    assert a[3][0] == 0 and ref[3][0] == 0    # no non-finite projections
    np.testing.assert_array_equal(a[0], b[0])
    err = np.abs(a[0] - ref[0]).max()
    print(f"beam with contacts, 40 steps: versioned vs colour launches {err:.3e}; launches per step "
          f"{max(a[2])} vs {min(ref[2])}")
    assert err <= 2e-6, err
    # one cooperative sweep per substep instead of 8 colours x 8 iterations + contacts
    assert max(a[2]) < 12 < min(ref[2])


def test_versioned_contacts_batch_equals_instances_alone(lib):
    insts = []
    for n, m in [(3, 4), (1, 1), (4, 3)]:
        X, tets, faces = G.grid_mesh(n, 2 * n, m, 0.01)
        insts.append((X, tets, faces))
    spheres = []
    for X, _, _ in insts:
        r = 0.4 * X[:, 0].max()
        spheres.append((np.array([[X[:, 0].max() / 2, X[:, 1].max() / 2, X[:, 2].max() + 0.9 * r]]), np.array([r])))
    kw = dict(num_iters=6, gs_variant=4)
    b = G.XPBDSolver(instances=[(X, t, f, 3e3, 0.45, 1000.0) for X, t, f in insts], **kw)
    b.fix_vertices(np.concatenate([X[:, 2] == 0 for X, _, _ in insts]))
    singles = []
    for (X, t, f) in insts:
        s = G.XPBDSolver(X, t, f, 3e3, 0.45, 1000.0, **kw)
        s.fix_vertices(X[:, 2] == 0)
        singles.append(s)
    for step in range(30):
        for k, (c, r) in enumerate(spheres):
            c2 = c + np.array([0, 0, -0.05]) * b.time
            b.set_spheres(c2, r, instance=k)
            singles[k].set_spheres(c2, r)
        b.step(1)
        for s in singles:
            s.step(1)
    xb = b.positions()
    off = 0
    ncon = 0
    for (X, _, _), s in zip(insts, singles):
        np.testing.assert_array_equal(xb[off:off + X.shape[0]], s.positions())
        ncon += len(s.collisions())
        off += X.shape[0]
        s.close()
    assert ncon > 0
    b.close()
