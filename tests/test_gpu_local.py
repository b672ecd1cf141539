"""Local collision iterations (num-local-collision-iters,
XPBDMeshObject.cpp:472-505 and :764-825) on the GPU against the FP64 oracle
run in the same order, on the small beam with the GPU's own contacts."""
import numpy as np
import pytest

import oracle as O
import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _beam():
    w = W.beam(nl=20, nw=4, nh=4, length=0.1)
    w.sphere_r = 0.02
    w.sphere_c0 = np.array([w.X[:, 0].max() / 2, w.X[:, 1].max() / 2, w.X[:, 2].max() + 0.02 - 0.002])
    return w


def test_local_order_is_a_valid_colouring(lib):
    w = _beam()
    s = W.make_solver(w, num_iters=4, num_local_collision_iters=2)
    order, off = s.local_order()
    np.testing.assert_array_equal(np.sort(order), np.arange(w.T))
    for c in range(len(off) - 1):
        tets = order[off[c]:off[c + 1]]
        assert np.all(np.diff(tets) > 0)  # ascending tet index within a colour
        v = w.tets[tets].ravel()
        assert len(np.unique(v)) == len(v)  # no shared vertex inside a colour
    s.close()
    plain = W.make_solver(w, num_iters=4)
    with pytest.raises(G.XPBDError):
        plain.local_order()
    plain.close()


@pytest.mark.parametrize("solver", [G.SOLVER_GAUSS_SEIDEL, G.SOLVER_JACOBI])
@pytest.mark.parametrize("ckind", [G.CONSTRAINT_COMBINED, G.CONSTRAINT_SEPARATE])
def test_local_iterations_match_fp64_oracle(lib, solver, ckind):
    w = _beam()
    if solver == G.SOLVER_JACOBI:
        w.nu = np.full(w.T, 0.3)  # the reference's plain-sum Jacobi diverges at nu = 0.49
    L = 3
    s = W.make_solver(w, num_iters=6, solver_type=solver, constraint_type=ckind, num_local_collision_iters=L)
    ref = W.make_solver(w, num_iters=6, solver_type=solver, constraint_type=ckind)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=6,
                 solver=O.JACOBI if solver == G.SOLVER_JACOBI else O.COLOURED_GS,
                 ckind=O.SEPARATE if ckind == G.CONSTRAINT_SEPARATE else O.COMBINED)
    o.set_fixed(w.fixed)
    if solver == G.SOLVER_GAUSS_SEIDEL:
        o.set_order(s.sweep_order())
    o.set_local_iterations(L, s.local_order()[0])
    for gpu in (s, ref):
        gpu.set_spheres(w.sphere_centre(0.0), [w.sphere_r])
        gpu.detect_collisions()
    rows = s.collisions()
    assert len(rows) > 0
    o.set_contacts(rows)
    for _ in range(8):
        for gpu in (s, ref):
            gpu.update()
            gpu.velocity_update()
        o.update()
        o.velocity_update()
    ext = float((w.X.max(0) - w.X.min(0)).max())
    err = np.abs(s.positions() - o.positions()).max()
    assert err <= 1e-4 * ext, err
    # the local passes changed the result
    assert np.abs(s.positions() - ref.positions()).max() > 1e-7
    s.close()
    ref.close()
    o.close()
