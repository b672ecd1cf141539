"""Learned warm start on the GPU: the tensor-core network (forward, gradient,
Adam) against the numpy oracle, the recorded training pairs against their
definition, the warm-started substep against the FP64 oracle's warm start,
and an A/B of the trained network against the plain start."""
import numpy as np
import pytest

import mlp_oracle as M
import oracle as O
import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _features(n, seed=0):
    """Rows shaped like the solver's: F near identity, alpha~ lambda O(1),
    log10(E)/5, nu, 1e3 dt, two zero pads."""
    rng = np.random.default_rng(seed)
    X = np.zeros((n, 16), np.float32)
    F = np.eye(3)[None] + 0.05 * rng.standard_normal((n, 3, 3))
    X[:, :9] = F.transpose(0, 2, 1).reshape(n, 9)
    X[:, 9:11] = rng.standard_normal((n, 2))
    X[:, 11] = rng.uniform(0.6, 1.0, n)
    X[:, 12] = rng.uniform(0.40, 0.49, n)
    X[:, 13] = 1.0
    return X


def _solver(n=4, **kw):
    X, tets, faces = G.grid_mesh(n, n, n, 1.0 / n)
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, dt=1e-3, num_iters=5, **kw)
    s.fix_vertices(X[:, 2] == 0)
    return s


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 40_000])
def test_forward_matches_oracle(lib, n):
    s = _solver()
    p = M.init_params(7)
    p[7] = np.array([0.3, -0.2], np.float32)
    s.set_mlp_params(M.flatten(p))
    X = _features(n, seed=n)
    out = s.mlp_forward(X)
    ref, _ = M.forward(p, X)
    scale = max(1.0, float(np.abs(ref).max()))
    err = np.abs(out - ref)
    # single BF16 rounding flips of hidden activations (2^-8 relative) bound
    # the element error; their mean stays far below it
    assert err.max() <= 2e-3 * scale, err.max()
    assert err.mean() <= 2e-4 * scale, err.mean()
    s.close()


def test_parameters_round_trip_and_init_is_seeded(lib):
    s = _solver()
    s.mlp_init(5)
    a = s.mlp_params()
    s.mlp_init(5)
    np.testing.assert_array_equal(a, s.mlp_params())
    W1 = M.unflatten(a)[0]
    assert np.all(W1[:, 14:] == 0) and np.isfinite(a).all()
    v = np.random.default_rng(1).standard_normal(G.MLP_PARAMS).astype(np.float32)
    s.set_mlp_params(v)
    np.testing.assert_array_equal(s.mlp_params(), v)
    with pytest.raises(RuntimeError):
        s.set_mlp_params(v[:-1])
    s.close()


@pytest.mark.parametrize("n", [200, 3000])
def test_gradient_matches_oracle(lib, n):
    """The GPU gradient against the oracle's model of the same precision
    (BF16 tensor-core operands), and against the exact FP64 gradient of the
    rounded forward pass (gradient check)."""
    s = _solver()
    p = M.init_params(11)
    p[1] = 0.1 * np.random.default_rng(2).standard_normal(64).astype(np.float32)
    s.set_mlp_params(M.flatten(p))
    X = _features(n, seed=3)
    Y = np.random.default_rng(4).standard_normal((n, 2)).astype(np.float32)
    loss, g = s.mlp_loss_grad(X, Y)
    ref_loss, ref_g = M.loss_and_grads(p, X, Y)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    _, exact_g = M.loss_and_grads(p, X, Y, rounding=True, round_grad=False)
    gl = M.unflatten(g)
    for k in range(8):
        nrm = np.linalg.norm(ref_g[k])
        assert np.linalg.norm(gl[k] - ref_g[k]) <= 1e-2 * nrm + 1e-7, (k, np.linalg.norm(gl[k] - ref_g[k]), nrm)
        nrm_e = np.linalg.norm(exact_g[k])
        assert np.linalg.norm(gl[k] - exact_g[k]) <= 3e-2 * nrm_e + 1e-7, k
    s.close()


def test_adam_matches_oracle(lib):
    s = _solver()
    p = M.init_params(2)
    s.set_mlp_params(M.flatten(p))
    rng = np.random.default_rng(9)
    m = [np.zeros(a.shape) for a in p]
    v = [np.zeros(a.shape) for a in p]
    q = p
    for t in (1, 2, 3):
        g = rng.standard_normal(G.MLP_PARAMS).astype(np.float32)
        s.mlp_adam_step(lr=1e-3, grad=g)
        q, m, v = M.adam_step(q, M.unflatten(g), m, v, t, lr=1e-3)
    np.testing.assert_allclose(s.mlp_params(), M.flatten(q), rtol=1e-5, atol=1e-7)
    s.close()


def test_device_gradient_feeds_adam(lib):
    """loss_grad leaves its gradient on the device; adam_step(None) uses it."""
    s = _solver()
    p = M.init_params(4)
    s.set_mlp_params(M.flatten(p))
    X = _features(500, seed=1)
    Y = np.ones((500, 2), np.float32)
    _, g = s.mlp_loss_grad(X, Y)
    s.mlp_adam_step(lr=1e-3)
    a = s.mlp_params()
    s.set_mlp_params(M.flatten(p))
    s.mlp_adam_step(lr=1e-3, grad=g)
    np.testing.assert_array_equal(a, s.mlp_params())
    s.close()


def test_recorded_pairs_match_their_definition(lib):
    """Features: F at the predicted positions (column-major), alpha~ lambda of
    the previous substep, log10(E)/5, nu, 1e3 dt. Targets: alpha~ lambda
    after the iterations."""
    w = W.cube(4, seed=1)
    s = W.make_solver(w, num_iters=5)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, num_iter=1)
    _, _, ad, ah, _ = o.tet_data()
    o.close()
    s.mlp_record(True)
    s.step(3)
    x = s.positions()
    v = s.velocities()
    lam_prev = s.lambdas()
    s.update()
    X, Y = s.mlp_samples()
    # predicted positions (XPBDMeshObject.cpp:449-456)
    xp = x + w.dt * v
    xp[:, 2] -= w.g * w.dt * w.dt
    e = w.tets
    Dm = np.stack([w.X[e[:, i]] - w.X[e[:, 3]] for i in range(3)], -1)
    Ds = np.stack([xp[e[:, i]] - xp[e[:, 3]] for i in range(3)], -1)
    F = Ds @ np.linalg.inv(Dm)
    np.testing.assert_allclose(X[:, :9], F.transpose(0, 2, 1).reshape(-1, 9), atol=1e-2, rtol=1e-2)
    dt2 = w.dt ** 2
    atd, ath = (ad / dt2).astype(np.float32), (ah / dt2).astype(np.float32)
    bf = lambda a: M.bf16(np.asarray(a, np.float32))
    np.testing.assert_allclose(X[:, 9], bf(atd * lam_prev[:, 0]), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(X[:, 10], bf(ath * lam_prev[:, 1]), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(X[:, 11], bf(np.log10(w.E) / 5), rtol=1e-6)
    np.testing.assert_allclose(X[:, 12], bf(w.nu), rtol=1e-6)
    np.testing.assert_allclose(X[:, 13], bf(np.full(w.T, w.dt * 1e3)), rtol=1e-6)
    assert np.all(X[:, 14:] == 0)
    lam = s.lambdas()
    np.testing.assert_allclose(Y[:, 0], atd * lam[:, 0], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(Y[:, 1], ath * lam[:, 1], rtol=1e-5, atol=1e-6)
    s.close()


@pytest.mark.parametrize("solver", [G.SOLVER_GAUSS_SEIDEL, G.SOLVER_JACOBI])
def test_previous_lambda_warm_start_matches_fp64_oracle(lib, solver):
    """XPBD_WARM_PREVIOUS against the oracle's warm-started update with the
    previous substep's multipliers: same keep/reject decisions, positions
    within the FP32 band."""
    w = W.cube(4, seed=2)
    s = W.make_solver(w, num_iters=6, solver_type=solver)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=6,
                 solver=O.JACOBI if solver == G.SOLVER_JACOBI else O.COLOURED_GS)
    o.set_fixed(w.fixed)
    o.set_positions(w.x0)
    if solver == G.SOLVER_GAUSS_SEIDEL:
        o.set_order(s.sweep_order())
    s.step(2)
    o.time_steps(2)
    s.set_warm_start(G.WARM_PREVIOUS)
    kept_ref = 0
    for _ in range(10):
        s.update()
        s.velocity_update()
        kept_ref += int(o.update_warm(o.lambdas()))
        o.velocity_update()
    kept, rejected = s.warm_start_stats()
    assert kept + rejected == 10
    assert kept == kept_ref
    err = np.abs(s.positions() - o.positions()).max()
    assert err <= 1e-4, err
    s.close()
    o.close()


@pytest.mark.parametrize("policy", [G.RESIDUAL_NEVER, G.RESIDUAL_EVERY_SUBSTEP, G.RESIDUAL_EVERY_ITERATION])
def test_rejected_warm_starts_reproduce_the_plain_solver(lib, policy):
    """A network whose prediction is rejected on every substep leaves the
    trajectory bit-identical to the plain start, and the residual history
    (record 0 = ||r(x_pred, 0)||) identical too."""
    w = W.cube(6, seed=3)
    plain = W.make_solver(w, num_iters=8, residual_policy=policy)
    warm = W.make_solver(w, num_iters=8, residual_policy=policy)
    p = M.init_params(0)
    p[7] = np.array([50.0, -50.0], np.float32)  # alpha~ lambda_0 far off: rejected
    warm.set_mlp_params(M.flatten(p))
    warm.set_warm_start(G.WARM_MLP)
    plain.step(15)
    warm.step(15)
    kept, rejected = warm.warm_start_stats()
    assert (kept, rejected) == (0, 15)
    np.testing.assert_array_equal(plain.positions(), warm.positions())
    if policy != G.RESIDUAL_NEVER:
        np.testing.assert_array_equal(plain.residual_history(), warm.residual_history())
    plain.close()
    warm.close()


def test_online_training_and_ab(lib, capsys):
    """Online training on the solver's own substeps lowers the loss; then an
    A/B on 20 further substeps reports the relative residual after the
    iterations with and without the learned warm start. The residual test
    guarantees the warm start never begins above the plain start."""
    w = W.cube(8, seed=4)
    kw = dict(num_iters=10, residual_policy=G.RESIDUAL_EVERY_SUBSTEP)
    s = W.make_solver(w, **kw)
    s.mlp_init(1)
    s.mlp_record(True)
    losses = []
    for _ in range(30):
        s.step(1)
        losses.append(s.mlp_train(epochs=4, batch=512, lr=3e-3))
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])
    params = s.mlp_params()
    x, v = s.positions(), s.velocities()
    res = {}
    for mode in (G.WARM_NONE, G.WARM_MLP):
        t = W.make_solver(w, **kw)
        t.set_positions(x)
        t.set_velocities(v)
        t.set_mlp_params(params)
        t.step(1)  # previous multipliers for the features
        t.set_warm_start(mode)
        rel = []
        for _ in range(20):
            t.step(1)
            h = t.residual_history()
            rel.append(h[-1] / h[0])
        res[mode] = (float(np.mean(rel)), t.warm_start_stats())
        t.close()
    kept, rejected = res[G.WARM_MLP][1]
    assert kept + rejected == 20
    with capsys.disabled():
        print(f"\nwarm-start A/B: plain rel. residual {res[G.WARM_NONE][0]:.3e}, learned {res[G.WARM_MLP][0]:.3e} "
              f"(kept {kept}, rejected {rejected}); training loss {losses[0]:.3e} -> {losses[-1]:.3e}")
    if kept == 0:
        assert res[G.WARM_MLP][0] == res[G.WARM_NONE][0]
    s.close()
