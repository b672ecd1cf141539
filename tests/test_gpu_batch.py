"""Batched instances (config 4): many independent objects in one context,
advanced by the same kernel launches."""
import numpy as np
import pytest

import oracle as O
import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _small_batch(n=5, seed=3):
    return W.batched(n=n, seed=seed, t_range=(300, 3000), iters=6)


def _drive_single(s, w, t):
    c, r = w.meta["spheres"]
    s.set_spheres(c + w.sphere_v * t, r)


def test_batch_offsets_and_sizes(lib):
    b = _small_batch()
    s = W.make_batch_solver(b)
    v, t, f = s.instance_offsets()
    assert s.n_instances == len(b.instances)
    np.testing.assert_array_equal(np.diff(v), [w.V for w in b.instances])
    np.testing.assert_array_equal(np.diff(t), [w.T for w in b.instances])
    np.testing.assert_array_equal(np.diff(f), [w.faces.shape[0] for w in b.instances])
    s.close()


def test_batched_equals_each_instance_alone(lib):
    """Gauss-Seidel is bit-reproducible and greedy colours of disjoint instances
    do not interact, so a batch reproduces every instance solved on its own."""
    b = _small_batch()
    s = W.make_batch_solver(b)
    singles = [W.make_solver(w) for w in b.instances]
    for step in range(25):
        W.drive_batch(s, b)
        s.step(1)
        for w, si in zip(b.instances, singles):
            _drive_single(si, w, si.time)
            si.step(1)
    xb = s.positions()
    v, _, _ = s.instance_offsets()
    ncont = len(s.collisions())
    assert ncont > 0
    for k, si in enumerate(singles):
        np.testing.assert_array_equal(xb[v[k]:v[k + 1]], si.positions())
        si.close()
    s.close()


def test_batched_instances_match_fp64_oracle(lib):
    b = _small_batch(n=3, seed=5)
    s = W.make_batch_solver(b)
    order = s.sweep_order()
    v, t, _ = s.instance_offsets()
    oracles = []
    for k, w in enumerate(b.instances):
        o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=w.iters, solver=O.COLOURED_GS)
        o.set_fixed(w.fixed)
        mine = order[(order >= t[k]) & (order < t[k + 1])] - t[k]
        o.set_order(mine)
        o.set_collision_rate(w.collision_rate)
        oracles.append(o)
    for step in range(20):
        W.drive_batch(s, b)
        s.step(1)
        for w, o in zip(b.instances, oracles):
            c, r = w.meta["spheres"]
            o.set_spheres(c + w.sphere_v * o.time, r)
            o.time_steps(1)
    xb = s.positions()
    for k, (w, o) in enumerate(zip(b.instances, oracles)):
        ext = float((w.X.max(0) - w.X.min(0)).max())
        err = np.abs(xb[v[k]:v[k + 1]] - o.positions()).max()
        # contacts are detected independently on both sides (FP32 vs FP64), so
        # a face right at the 1e-4 threshold may differ; 1e-3 x extent bound
        assert err <= 1e-3 * ext, (k, err)
    s.close()


def test_batch_full_size_runs(lib):
    """256 instances, ~6.5M tets: a few steps stay finite with fixed bottoms."""
    b = W.batched()
    s = W.make_batch_solver(b)
    for _ in range(3):
        W.drive_batch(s, b)
        s.step(1)
    s.synchronize()
    x = s.positions()
    assert np.isfinite(x).all()
    fixed = np.concatenate([w.fixed for w in b.instances])
    X = np.concatenate([w.X for w in b.instances])
    np.testing.assert_allclose(x[fixed], X[fixed], atol=1e-7)
    nonfinite, _ = s.health()
    assert nonfinite == 0
    s.close()


def test_l2_stream_priority_leaves_results_unchanged(lib):
    """gs_l2_stream only sets the L2 eviction priority of the sweep's streamed
    records (evict-first or normal): every mode gives the same positions bit
    for bit, on a batch whose sweep streams its patch records (not resident)."""
    b = _small_batch(n=8, seed=7)
    xs = []
    for mode in (-1, 0, 1):
        s = W.make_batch_solver(b, gs_l2_stream=mode)
        for _ in range(6):
            W.drive_batch(s, b)
            s.step(1)
        xs.append(s.positions())
        s.close()
    np.testing.assert_array_equal(xs[0], xs[1])
    np.testing.assert_array_equal(xs[0], xs[2])
    with pytest.raises(G.XPBDError):
        W.make_batch_solver(b, gs_l2_stream=2)


@pytest.mark.parametrize("solver,ncand",[(G.SOLVER_GAUSS_SEIDEL, 48), (G.SOLVER_JACOBI, 12)])
def test_autotuner_times_every_candidate_and_keeps_the_fastest(lib, solver, ncand):
    b = _small_batch(n=3)
    inst = [(w.X, w.tets, w.faces, w.E, w.nu, w.rho) for w in b.instances]
    best, results = G.autotune(inst, trial_steps=3, solver_type=solver, num_iters=5)
    assert len(results) == ncand and all(r["ms_per_step"] > 0 for r in results)
    fastest = min(results, key=lambda r: r["ms_per_step"])
    keys = ["gs_patch_tets", "gs_variant", "gs_min_blocks", "use_pdl"] if solver == G.SOLVER_GAUSS_SEIDEL \
        else ["block_size", "jacobi_variant", "use_pdl"]
    for k in keys:
        assert getattr(best, k) == fastest[k]
    # the chosen configuration runs
    s = G.XPBDSolver(instances=inst, num_iters=5, solver_type=solver,
                     **{k: getattr(best, k) for k in ["gs_patch_tets", "gs_variant", "gs_min_blocks", "block_size",
                                                      "jacobi_variant", "use_pdl"]})
    s.step(2)
    s.synchronize()
    s.close()


def test_instance_latency_stamps(lib):
    """Per-instance completion times of the persistent sweep: one per
    instance, inside the substep, spread over it, and the stamps change no
    result (a run without them ends bit-identical)."""
    b = _small_batch(n=6, seed=4)
    s = W.make_batch_solver(b, gs_variant=4)
    plain = W.make_batch_solver(b, gs_variant=4)
    with pytest.raises(G.XPBDError):
        s.instance_latencies()  # nothing stamped yet
    s.set_latency_stamps(True)
    for _ in range(6):
        for x in (s, plain):
            W.drive_batch(x, b)
            x.step(1)
        ms, batch_ms = s.instance_latencies()
        assert ms.shape == (len(b.instances),)
        assert np.all(ms > 0) and np.all(ms <= batch_ms + 1e-6), (ms, batch_ms)
    np.testing.assert_array_equal(s.positions(), plain.positions())
    s.set_latency_stamps(False)
    W.drive_batch(s, b)
    s.step(1)
    with pytest.raises(G.XPBDError):
        s.instance_latencies()
    s.close()
    plain.close()


def test_latency_stamps_need_the_versioned_sweep(lib):
    b = _small_batch(n=2, seed=4)
    s = W.make_batch_solver(b, gs_variant=1)
    with pytest.raises(G.XPBDError):
        s.set_latency_stamps(True)
    s.close()
