"""Edge cases of the solver path: the smallest mesh (one tet, the reference's
resource/general/single.msh case), zero iterations, and ragged batches in
which a one-tet instance sits beside instances a thousand times larger."""
import numpy as np
import pytest

import oracle as O
import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _one_tet():
    X = 0.1 * np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    tets = np.array([[0, 1, 2, 3]], dtype=np.int32)
    faces = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]], dtype=np.int32)
    return X, tets, faces


@pytest.mark.parametrize("solver,var", [(G.SOLVER_JACOBI, 0), (G.SOLVER_GAUSS_SEIDEL, 0),
                                        (G.SOLVER_GAUSS_SEIDEL, 1), (G.SOLVER_GAUSS_SEIDEL, 2),
                                        (G.SOLVER_GAUSS_SEIDEL, 3), (G.SOLVER_GAUSS_SEIDEL, 4)])
def test_single_tet_matches_fp64_oracle(lib, solver, var):
    """One tet hanging from a fixed vertex under gravity, 10 iterations per
    step, 60 steps: every sweep variant (one patch, one task, one warp) and
    Jacobi stay within 1e-4 of the extent of the FP64 oracle."""
    X, tets, faces = _one_tet()
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, num_iters=10, solver_type=solver, gs_variant=var)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, num_iter=10,
                 solver=O.JACOBI if solver == G.SOLVER_JACOBI else O.COLOURED_GS, precision=64)
    if solver == G.SOLVER_GAUSS_SEIDEL:
        o.set_order(s.sweep_order())
    fixed = np.array([False, False, False, True])
    s.fix_vertices(fixed)
    o.set_fixed(fixed)
    s.step(60)
    o.time_steps(60)
    x, xo = s.positions(), o.positions()
    assert np.abs(x - xo).max() <= 1e-4 * 0.1
    # it moved: the free vertices fell and the tet stretched toward vertex 3
    assert x[:3, 2].max() < X[:3, 2].max() - 1e-4
    # fixed: exactly its (FP32) rest position
    np.testing.assert_array_equal(x[3], X[3].astype(np.float32))
    s.close()
    o.close()


def test_zero_iterations_is_semi_implicit_free_fall(lib):
    """num_iters = 0: a step is the inertial prediction and the velocity
    update only, x_n = x_0 + dt sum v_k with v_k = v_0 - k g dt (FP32), and
    fixed vertices stay put."""
    w = W.cube(n=3)
    s = G.XPBDSolver(w.X, w.tets, None, 3e3, 0.45, 1000.0, num_iters=0)
    s.fix_vertices(w.fixed)
    n, dt, g = 25, 1e-3, 9.81
    s.step(n)
    x = s.positions()
    exp = w.X.copy()
    exp[:, 2] -= g * dt * dt * n * (n + 1) / 2
    free = ~w.fixed
    # FP32: with v = (x - x_prev) / dt the positions follow x' = 2x - x_prev + dz,
    # which carries each step's rounding (ulp(1) / 2) into every later step:
    # at most n^2 / 2 of them after n steps, 2e-5 here
    eps = np.finfo(np.float32).eps / 2
    np.testing.assert_allclose(x[free], exp[free], rtol=0, atol=n * n / 2 * eps)
    # the velocity is a difference of positions near 1 over dt
    np.testing.assert_allclose(s.velocities()[free, 2], -n * g * dt, rtol=0, atol=4 * n * eps / dt)
    np.testing.assert_array_equal(x[w.fixed], w.X[w.fixed].astype(np.float32))
    s.close()


def _ragged_instances(with_faces):
    X1, t1, f1 = _one_tet()
    X2, t2, f2 = G.grid_mesh(6, 6, 6, 0.1 / 6)        # 1,080 tets
    X3, t3, f3 = G.grid_mesh(40, 4, 4, 0.5 / 40)      # 3,200 tets
    X4, t4, f4 = G.grid_mesh(1, 1, 2, 0.05)           # 10 tets
    inst = []
    for X, t, f, E in [(X1, t1, f1, 3e3), (X2, t2, f2, 1e4), (X3, t3, f3, 5e3), (X4, t4, f4, 2e3)]:
        inst.append((X, t, f if with_faces else None, E, 0.45, 1000.0))
    return inst


@pytest.mark.parametrize("solver,var,with_faces", [(G.SOLVER_GAUSS_SEIDEL, 4, False),
                                                   (G.SOLVER_GAUSS_SEIDEL, 2, False),
                                                   (G.SOLVER_GAUSS_SEIDEL, 0, True),
                                                   (G.SOLVER_JACOBI, 0, True)])
def test_ragged_batch_reproduces_each_instance_alone(lib, solver, var, with_faces):
    """Instances of 1 to 3,200 tets in one context: each one's trajectory is
    that of the same instance solved alone (Gauss-Seidel bit for bit, with the
    one-launch sweeps over all instances or the colour launches; Jacobi within
    FP32 atomic-order rounding)."""
    inst = _ragged_instances(with_faces)
    kw = dict(num_iters=6, solver_type=solver, gs_variant=var)
    b = G.XPBDSolver(instances=inst, **kw)
    singles = [G.XPBDSolver(*i, **kw) for i in inst]
    fixed = [i[0][:, 2] == i[0][:, 2].min() for i in inst]
    b.fix_vertices(np.concatenate(fixed))
    for s1, f in zip(singles, fixed):
        s1.fix_vertices(f)
    b.step(12)
    xb = b.positions()
    voff, _, _ = b.instance_offsets()
    for k, s1 in enumerate(singles):
        s1.step(12)
        xs = s1.positions()
        part = xb[voff[k]:voff[k + 1]]
        if solver == G.SOLVER_GAUSS_SEIDEL:
            np.testing.assert_array_equal(part, xs)
        else:
            assert np.abs(part - xs).max() <= 1e-6
        s1.close()
    b.close()


def test_meshes_the_reference_cannot_solve_are_refused(lib):
    """Inputs for which the reference's setup divides by zero or takes the
    log of a negative number (ElementConstraint.hpp:23-51, ElasticMaterial.hpp:31-32)
    are refused with XPBD_ERR_INVALID at creation: a tet whose rest vertices
    are coplanar, a non-finite vertex, E <= 0, nu outside (-1, 0.5), density <= 0."""
    X, tets, _ = _one_tet()
    flat = X.copy()
    flat[3] = [0.05, 0.05, 0.0]                 # in the plane of the other three
    nan = X.copy()
    nan[2, 1] = np.nan
    cases = [(flat, 3e3, 0.45, 1000.0), (nan, 3e3, 0.45, 1000.0), (X, 0.0, 0.45, 1000.0),
             (X, 3e3, 0.5, 1000.0), (X, 3e3, 0.45, -1.0)]
    for Xc, E, nu, rho in cases:
        with pytest.raises(G.XPBDError) as e:
            G.XPBDSolver(Xc, tets, None, E, nu, rho)
        assert e.value.status == G.XPBD_ERR_INVALID
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0)     # the valid tet is accepted
    s.close()


def test_a_wait_that_runs_out_reports_timeout_and_the_context_recovers(lib):
    """The versioned sweep's waits are bounded. A vertex whose due version is
    never written (the test hook) makes its patches' waits give up after 4,096
    polls; the abort flag sends every other waiter home, the kernel returns,
    xpbd_synchronize reports XPBD_ERR_TIMEOUT and xpbd_health clears it. With
    the tables restored the same context steps on and matches a fresh one."""
    w = W.cube(n=5)
    s = G.XPBDSolver(w.X, w.tets, None, 3e3, 0.45, 1000.0, num_iters=6)
    s.fix_vertices(w.fixed)
    s.set_positions(w.x0)
    s.step(1)
    s.synchronize()
    s.debug_stall_vertex(int(np.nonzero(~w.fixed)[0][7]), 4096)
    s.step(1)
    with pytest.raises(G.XPBDError) as e:
        s.synchronize()
    assert e.value.status == G.XPBD_ERR_TIMEOUT
    s.health()                     # clears the counters
    s.debug_stall_vertex(-1)
    # from one state, the recovered context and a fresh one take the same 3 steps
    f = G.XPBDSolver(w.X, w.tets, None, 3e3, 0.45, 1000.0, num_iters=6)
    f.fix_vertices(w.fixed)
    out = []
    for c in (s, f):
        c.set_positions(w.x0)
        c.set_velocities(np.zeros_like(w.X))
        c.step(3)
        c.synchronize()
        assert c.health()[0] == 0
        out.append(c.positions())
        c.close()
    np.testing.assert_array_equal(out[0], out[1])
