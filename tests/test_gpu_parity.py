"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on the
same seeded inputs.

Tolerances (max vertex error against the FP64 oracle run in the same order)
  * short horizons (20 steps): <= 1e-4 x mesh extent, the benchmark spec's bound;
  * long horizons (100 steps): <= max(1e-4 x extent, 3 x band32), where band32
    is the deviation of the FP32 oracle (an exact FP32 restatement) from the
    FP64 oracle on the same trajectory. On soft, large-deformation meshes FP32
    rounding alone moves vertices by more than 1e-4 x extent over 100 steps
    (1.4e-4 Jacobi, 3.4e-4 coloured Gauss-Seidel on the 10^3 cube), so the
    device is held to the accuracy FP32 can reach on that trajectory;
  * single projections vs the FP32 oracle: 1e-4 of the update.
"""
import numpy as np
import pytest

import oracle as O
import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _extent(X):
    return float((X.max(0) - X.min(0)).max())


def _pair(X, tets, faces, E, nu, rho, solver, iters, dt=1e-3, g=9.81, ckind=G.CONSTRAINT_COMBINED, precision=64,
          with_faces=False, **kw):
    s = G.XPBDSolver(X, tets, faces if with_faces else None, E, nu, rho, dt=dt, g_accel=g, num_iters=iters,
                     solver_type=solver, constraint_type=ckind, **kw)
    o = O.Oracle(X, tets, faces, E, nu, rho, dt=dt, g=g, num_iter=iters,
                 solver=O.JACOBI if solver == G.SOLVER_JACOBI else O.COLOURED_GS,
                 ckind=O.SEPARATE if ckind == G.CONSTRAINT_SEPARATE else O.COMBINED, precision=precision)
    if solver == G.SOLVER_GAUSS_SEIDEL:
        o.set_order(s.sweep_order())  # replay the GPU's colour/patch order
    return s, o


def _noisy_cube(n=4, seed=1, noise=2e-3):
    X, tets, faces = G.grid_mesh(n, n, n, 1.0 / n)
    x0 = X + np.random.default_rng(seed).uniform(-noise, noise, X.shape)
    return X, tets, faces, x0


@pytest.mark.parametrize("solver", [G.SOLVER_JACOBI, G.SOLVER_GAUSS_SEIDEL])
@pytest.mark.parametrize("ckind", [G.CONSTRAINT_COMBINED, G.CONSTRAINT_SEPARATE])
def test_single_update_matches_fp32_oracle(lib, solver, ckind):
    X, tets, faces, x0 = _noisy_cube(3, seed=2, noise=0.02)
    s, o = _pair(X, tets, faces, 5e3, 0.4, 1000.0, solver, 1, ckind=ckind, precision=32)
    s.set_positions(x0); o.set_positions(x0)
    s.update(); o.update()
    xs, xo = s.positions(), o.positions()
    scale = np.abs(xo - x0).max()
    assert np.abs(xs - xo).max() <= 1e-4 * scale + 1e-7
    np.testing.assert_allclose(s.lambdas(), o.lambdas(), rtol=1e-3, atol=1e-6 * np.abs(o.lambdas()).max())
    s.close()


def _oracle_pair(X, tets, faces, E, nu, rho, solver, iters, gpu=None, **kw):
    """FP32 and FP64 oracles; for Gauss-Seidel they replay the GPU's sweep order."""
    def mk(prec):
        o = O.Oracle(X, tets, faces, E, nu, rho, num_iter=iters,
                     solver=O.JACOBI if solver == G.SOLVER_JACOBI else O.COLOURED_GS, precision=prec, **kw)
        if solver == G.SOLVER_GAUSS_SEIDEL:
            o.set_order(gpu.sweep_order())
        return o
    return mk(32), mk(64)


@pytest.mark.parametrize("solver,cap,var", [(G.SOLVER_JACOBI, 0, 0), (G.SOLVER_GAUSS_SEIDEL, 5, 0),
                                            (G.SOLVER_GAUSS_SEIDEL, 1, 0), (G.SOLVER_GAUSS_SEIDEL, 5, 1),
                                            (G.SOLVER_GAUSS_SEIDEL, 5, 2), (G.SOLVER_GAUSS_SEIDEL, 2, 2),
                                            (G.SOLVER_GAUSS_SEIDEL, 5, 3), (G.SOLVER_GAUSS_SEIDEL, 5, 4),
                                            (G.SOLVER_GAUSS_SEIDEL, 2, 4)])
def test_cube_trajectory_matches_fp64_oracle(lib, solver, cap, var):
    """Config-1 mesh (10^3 hexes, bottom fixed, seeded noise): 20 steps at the
    spec bound, then 100 steps within the FP32 band. Gauss-Seidel runs
    with hex patches (cap 5), per-tet colouring (cap 1), and every sweep
    kernel variant (registers, shared-memory staging, dataflow on task
    counters, dataflow on vertex versions)."""
    w = W.cube()
    s = G.XPBDSolver(w.X, w.tets, None, w.E, w.nu, w.rho, num_iters=10, solver_type=solver, gs_patch_tets=cap,
                     gs_variant=var)
    o32, o64 = _oracle_pair(w.X, w.tets, w.faces, w.E, w.nu, w.rho, solver, 10, gpu=s)
    s.set_positions(w.x0)
    s.fix_vertices(w.fixed)
    for o in (o32, o64):
        o.set_positions(w.x0); o.set_fixed(w.fixed)
    ext = _extent(w.X)
    s.step(20); o32.time_steps(20); o64.time_steps(20)
    err20 = np.abs(s.positions() - o64.positions()).max()
    assert err20 <= 1e-4 * ext, err20
    s.step(80); o32.time_steps(80); o64.time_steps(80)
    band = np.abs(o32.positions() - o64.positions()).max()
    err = np.abs(s.positions() - o64.positions()).max()
    assert err <= max(1e-4 * ext, 3 * band), (err, band)
    vt = np.abs(s.velocities() - o64.velocities()).max()
    assert vt <= max(1e-4 * ext, 3 * band) / w.dt
    # fixed vertices are exactly back at their previous positions
    np.testing.assert_array_equal(s.positions()[w.fixed], s.prev_positions()[w.fixed])
    s.close()


def _patches(tets, cap, max_verts=8):
    """Independent restatement of the library's patch rule: runs of
    consecutive tets, each sharing a vertex with the run, at most `cap` tets
    and `max_verts` vertices."""
    runs, cur, verts = [], [], []
    for t, e in enumerate(tets):
        fresh = [v for v in e if v not in verts]
        if cur and (len(cur) == cap or len(fresh) == 4 or len(verts) + len(fresh) > max_verts):
            runs.append(cur); cur, verts = [], []
            fresh = list(e)
        cur.append(t); verts.extend(fresh)
    runs.append(cur)
    return runs


@pytest.mark.parametrize("cap", [1, 5])
def test_gs_sweep_order_is_patch_colouring(lib, cap):
    w = W.cube(n=6)
    s = G.XPBDSolver(w.X, w.tets, None, w.E, w.nu, w.rho, solver_type=G.SOLVER_GAUSS_SEIDEL, gs_patch_tets=cap)
    nt, _, col = s.colours()
    order = s.sweep_order()
    runs = _patches(w.tets, cap)
    assert sorted(order.tolist()) == list(range(w.T))
    if cap == 5:
        assert all(len(r) == 5 for r in runs) and nt == 8  # hex patches of the grid: 8 colours
    # colours are non-decreasing along the sweep, each patch keeps one colour
    assert np.all(np.diff(col[order]) >= 0)
    for r in runs:
        assert len(set(col[r])) == 1
    # patches of one colour share no vertex
    for c in range(nt):
        vs = [set(w.tets[r].ravel()) for r in runs if col[r[0]] == c]
        allv = [v for st in vs for v in st]
        assert len(allv) == len(set(allv))
    s.close()


@pytest.mark.parametrize("solver,var", [(G.SOLVER_JACOBI, 0), (G.SOLVER_GAUSS_SEIDEL, 0),
                                        (G.SOLVER_GAUSS_SEIDEL, 1)])
def test_separate_constraints_trajectory(lib, solver, var):
    X, tets, faces, x0 = _noisy_cube(4, seed=3)
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, num_iters=8, solver_type=solver,
                     constraint_type=G.CONSTRAINT_SEPARATE, gs_variant=var)
    o32, o64 = _oracle_pair(X, tets, faces, 3e3, 0.45, 1000.0, solver, 8, gpu=s, ckind=O.SEPARATE)
    fixed = X[:, 2] == 0
    s.set_positions(x0); s.fix_vertices(fixed)
    for o in (o32, o64):
        o.set_positions(x0); o.set_fixed(fixed)
    s.step(50); o32.time_steps(50); o64.time_steps(50)
    band = np.abs(o32.positions() - o64.positions()).max()
    err = np.abs(s.positions() - o64.positions()).max()
    assert err <= max(1e-4 * _extent(X), 3 * band), (err, band)
    s.close()


@pytest.mark.parametrize("solver", [G.SOLVER_JACOBI, G.SOLVER_GAUSS_SEIDEL])
def test_residual_history_and_queries(lib, solver):
    X, tets, faces, x0 = _noisy_cube(4, seed=4, noise=5e-3)
    s, o = _pair(X, tets, faces, 2e4, 0.45, 1000.0, solver, 6, residual_policy=G.RESIDUAL_EVERY_ITERATION)
    fixed = X[:, 2] == 0
    for m in (s, o):
        m.set_positions(x0)
    s.fix_vertices(fixed); o.set_fixed(fixed)
    s.step(3); o.time_steps(3, record=True)
    hs, ho = s.residual_history(), o.res_history()
    assert hs.shape == ho.shape == (7,)
    np.testing.assert_allclose(hs, ho, rtol=2e-3, atol=1e-6 * ho[0])
    # constraint residual vector (stored at the end of solve, reference order)
    r_gpu = s.constraint_residual()
    assert np.isclose(np.linalg.norm(r_gpu), hs[-1], rtol=1e-3)
    # exact residual and energy at the current state
    a, rel = s.residual()
    ref = o.residual_norm()
    assert np.isclose(a, ref, rtol=5e-3, atol=1e-5 * ho[0])
    assert 0 <= rel < 1.5
    e_s, e_o = s.strain_energy(), o.strain_energy()
    assert np.isclose(e_s, e_o, rtol=1e-3)
    np.testing.assert_allclose(s.lambdas(), o.lambdas(), rtol=5e-3, atol=1e-3 * np.abs(o.lambdas()).max())
    s.close()


def test_gather_variant_is_deterministic_and_matches_atomic(lib):
    w = W.cube(n=6)
    runs = []
    for variant in (G.JACOBI_GATHER, G.JACOBI_GATHER, G.JACOBI_ATOMIC):
        s = W.make_solver(w, num_iters=5, solver_type=G.SOLVER_JACOBI, jacobi_variant=variant)
        s.step(20)
        runs.append(s.positions())
        s.close()
    np.testing.assert_array_equal(runs[0], runs[1])
    assert np.abs(runs[0] - runs[2]).max() < 1e-6


@pytest.mark.parametrize("solver,var", [(G.SOLVER_JACOBI, 0), (G.SOLVER_GAUSS_SEIDEL, 0),
                                        (G.SOLVER_GAUSS_SEIDEL, 1), (G.SOLVER_GAUSS_SEIDEL, 2),
                                        (G.SOLVER_GAUSS_SEIDEL, 4)])
def test_graph_and_direct_launch_agree(lib, solver, var):
    w = W.cube(n=5)
    out = []
    for graphs in (1, 0):
        s = W.make_solver(w, num_iters=4, solver_type=solver, use_graphs=graphs,
                          jacobi_variant=G.JACOBI_GATHER, gs_variant=var)
        s.step(15)
        out.append(s.positions())
        nonfinite, _ = s.health()
        assert nonfinite == 0
        s.close()
    assert np.abs(out[0] - out[1]).max() <= 1e-6


def _beam_small():
    w = W.beam(nl=20, nw=4, nh=4, length=0.1)
    w.sphere_r = 0.02
    w.sphere_c0 = np.array([w.X[:, 0].max() / 2, w.X[:, 1].max() / 2, w.X[:, 2].max() + 0.02 - 0.002])
    return w


def test_collision_detection_matches_fp32_oracle(lib):
    w = _beam_small()
    s = W.make_solver(w, num_iters=1)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, precision=32)
    x = w.X.copy()
    x[:, 2] -= 0.5e-3 * np.sin(np.pi * x[:, 1] / x[:, 1].max())  # a sagged, non-grid state
    s.set_positions(x); o.set_positions(x)
    c = w.sphere_centre(0.0)
    s.set_spheres(c, [w.sphere_r]); o.set_spheres(c, [w.sphere_r])
    s.detect_collisions()
    nref = o.detect()
    cg, co = s.collisions(), o.contacts()
    assert nref > 0
    fg = {int(r[1]): r for r in cg}
    fo = {int(r[1]): r for r in co}
    common = set(fg) & set(fo)
    # threshold decisions may flip only for faces right at the 1e-4 cut
    assert len(set(fg) ^ set(fo)) <= max(1, nref // 50)
    for f in common:
        np.testing.assert_allclose(fg[f][2:11], fo[f][2:11], atol=2e-5)
    s.close()


@pytest.mark.parametrize("solver", [G.SOLVER_JACOBI, G.SOLVER_GAUSS_SEIDEL])
def test_beam_trajectory_with_injected_contacts(lib, solver):
    """Physics parity with contacts: the GPU's own detections are fed to the
    FP64 oracle, so detection threshold flips cannot mask projection errors.
    The reference's un-averaged Jacobi diverges on the nu = 0.49 beam (both here
    and in the oracle), and with overlapping face contacts it diverges after
    ~40 steps even at nu = 0.3; the Jacobi case runs 30 steps at nu = 0.3
    (two detections), the Gauss-Seidel case 60 steps on the beam material."""
    w = _beam_small()
    nsteps = 60
    if solver == G.SOLVER_JACOBI:
        w.nu = np.full(w.T, 0.3)
        nsteps = 30
    s = W.make_solver(w, num_iters=10, solver_type=solver)
    oracles = _oracle_pair(w.X, w.tets, w.faces, w.E, w.nu, w.rho, solver, 10, gpu=s, dt=w.dt, g=w.g)
    for o in oracles:
        o.set_fixed(w.fixed)
    t, last, interval = 0.0, 0.0, 1.0 / w.collision_rate
    ncontacts = 0
    for k in range(nsteps):
        if t - last > interval:
            s.set_spheres(w.sphere_centre(t), [w.sphere_r])
            s.detect_collisions()
            rows = s.collisions()
            ncontacts += len(rows)
            for o in oracles:
                o.set_contacts(rows)
        s.update(); s.velocity_update()
        for o in oracles:
            o.update(); o.velocity_update()
        if t - last > interval:
            last = t
        t += w.dt
    assert ncontacts > 0
    o32, o64 = oracles
    band = np.abs(o32.positions() - o64.positions()).max()
    err = np.abs(s.positions() - o64.positions()).max()
    assert np.isfinite(err) and err <= max(1e-4 * _extent(w.X), 3 * band), (err, band)
    s.close()


def test_step_loop_detection_cadence(lib):
    """xpbd_step runs detection on the reference's strict cadence; the built-in
    loop equals the manual detect/update/velocity loop."""
    w = _beam_small()
    # Gauss-Seidel: contacts update in place, so both loops are bit-reproducible
    a = W.make_solver(w, num_iters=5, solver_type=G.SOLVER_GAUSS_SEIDEL)
    b = W.make_solver(w, num_iters=5, solver_type=G.SOLVER_GAUSS_SEIDEL)
    t, last, interval = 0.0, 0.0, 1.0 / w.collision_rate
    for k in range(35):
        a.set_spheres(w.sphere_centre(a.time), [w.sphere_r])
        a.step(1)
        if t - last > interval:
            b.set_spheres(w.sphere_centre(t), [w.sphere_r])
            b.detect_collisions()
        b.update(); b.velocity_update()
        if t - last > interval:
            last = t
        t += w.dt
    assert abs(a.time - t) == 0.0
    np.testing.assert_array_equal(a.positions(), b.positions())
    a.close(); b.close()


def test_coloured_gs_contacts_match_oracle_order(lib):
    w = _beam_small()
    s = W.make_solver(w, num_iters=6, solver_type=G.SOLVER_GAUSS_SEIDEL)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, num_iter=6, solver=O.COLOURED_GS)
    o.set_order(s.sweep_order())
    o.set_fixed(w.fixed)
    s.set_spheres(w.sphere_centre(0.0), [w.sphere_r])
    s.detect_collisions()
    o.set_contacts(s.collisions())
    for _ in range(5):
        s.update(); s.velocity_update(); o.update(); o.velocity_update()
    assert np.abs(s.positions() - o.positions()).max() <= 1e-4 * _extent(w.X)


def test_add_static_collision_api(lib):
    X, tets, faces, x0 = _noisy_cube(3, seed=5)
    s = G.XPBDSolver(X, tets, faces, 3e3, 0.45, 1000.0, num_iters=4, solver_type=G.SOLVER_JACOBI)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, num_iter=4, solver=O.JACOBI)
    # a plane contact pushing the bottom faces up by 1 mm
    bottom = [f for f in range(len(faces)) if np.all(X[faces[f], 2] == 0)]
    rows = []
    for f in bottom:
        p = X[faces[f]].mean(0) + np.array([0, 0, 1e-3])
        n = np.array([0.0, 0.0, 1.0])
        s.add_static_collision(f, 1 / 3, 1 / 3, 1 / 3, p, n)
        rows.append([0, f, 1 / 3, 1 / 3, 1 / 3, *p, *n, 0])
    o.set_contacts(np.array(rows))
    s.update(); o.update()
    assert np.abs(s.positions() - o.positions()).max() < 1e-6
    assert len(s.collisions()) == len(bottom)
    s.clear_collisions()
    assert len(s.collisions()) == 0
    s.close()


def test_kinematic_block_matches_oracle(lib):
    w = W.block(n=6, iters=8)
    s = W.make_solver(w)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=8, solver=O.COLOURED_GS)
    o.set_order(s.sweep_order())
    o.set_fixed(w.fixed)
    o.set_kinematic_group(w.kin_idx)
    for k in range(40):
        off = w.kin_offset(k + 1)
        s.set_kinematic_offset(off); o.set_kinematic_offset(off)
        s.step(1); o.time_steps(1)
    xs = s.positions()
    assert np.abs(xs - o.positions()).max() <= 1e-4 * _extent(w.X)
    np.testing.assert_allclose(xs[w.kin_idx], w.X[w.kin_idx] + w.kin_offset(40), atol=1e-6)
    s.close()


def test_health_counts_degenerate_elements(lib):
    X, tets, faces = G.grid_mesh(2, 2, 2, 0.5)
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, num_iters=1, solver_type=G.SOLVER_JACOBI, g_accel=0.0)
    x = X.copy()
    x[:, 2] *= 1e-4  # flatten: every tet has |det F| ~ 1e-4
    s.set_positions(x)
    s.update()
    nonfinite, degenerate = s.health()
    assert degenerate > 0 and nonfinite == 0
    assert np.isfinite(s.positions()).all()
    s.close()


def test_residual_reductions_are_fp64(lib):
    """Per-tet E over six decades spreads the squared residual terms over
    many orders of magnitude. The last history entry reduces the FP64 terms
    of the state after the last sweep; the per-constraint vector read back
    holds the same terms rounded to FP32, so its FP64 norm differs from the
    entry by at most that rounding, 2^-24 relative. A reduction with FP32
    partial sums would miss the bound by about an order of magnitude."""
    X, tets, faces, x0 = _noisy_cube(6, seed=5, noise=5e-3)
    E = np.exp(np.random.default_rng(9).uniform(np.log(1e2), np.log(1e8), len(tets)))
    s = G.XPBDSolver(X, tets, None, E, 0.45, 1000.0, num_iters=4, residual_policy=G.RESIDUAL_EVERY_ITERATION)
    s.fix_vertices(X[:, 2] == 0)
    s.set_positions(x0)
    s.step(2)
    r = s.constraint_residual()
    ref = float(np.sqrt(np.sum(r.astype(np.float64) ** 2)))
    hs = s.residual_history()
    assert ref > 0 and np.abs(r).max() / np.abs(r[r != 0]).min() > 1e4
    assert abs(hs[-1] - ref) <= 2.0 ** -24 * ref, (hs[-1], ref)
    s.close()


def test_versioned_sweep_careful_pass_equals_colour_launches(lib):
    """The versioned sweep projects a patch in one straight FP32 pass and
    redoes it from the task's start with the per-tet FP64 guard when any of
    its tets is near-degenerate; the colour launches guard tet by tet. A mesh
    whose top layer is squashed flat (|det F| ~ 1e-4 there) takes both paths
    and must end bit-identical, with the same degenerate count."""
    X, tets, faces = G.grid_mesh(6, 6, 6, 1.0 / 6)
    x = X.copy()
    top = X[:, 2] > 1.0 - 1e-9
    x[top, 2] = 1.0 - 1.0 / 6 + 1e-4 / 6  # the top layer of hexes nearly flat
    out = []
    for var in (0, 4):
        s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, num_iters=6, gs_variant=var)
        s.fix_vertices(X[:, 2] == 0)
        s.set_positions(x)
        s.step(5)
        s.synchronize()
        out.append((s.positions(), s.lambdas(), s.health()))
        s.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2][1] > 0 and out[0][2] == out[1][2], (out[0][2], out[1][2])


def test_invalid_inputs_return_status(lib):
    X, tets, faces = G.grid_mesh(2, 2, 2, 0.5)
    bad = tets.copy()
    bad[0, 0] = 10_000
    with pytest.raises(G.XPBDError) as e:
        G.XPBDSolver(X, bad, None)
    assert e.value.status == G.XPBD_ERR_INVALID
    s = G.XPBDSolver(X, tets, faces)
    with pytest.raises(G.XPBDError) as e:
        s.set_spheres(np.zeros((20, 3)), np.ones(20))
    assert e.value.status == G.XPBD_ERR_INVALID
    with pytest.raises(G.XPBDError):
        s.set_kinematic_group([0, 10_000])
    s.close()


# ---- full-size workloads: size-independent properties ----

def test_block_full_size_properties(lib):
    w = W.block()
    s = W.make_solver(w, residual_policy=G.RESIDUAL_EVERY_ITERATION)
    for k in range(3):
        W.drive_gpu(s, w, k + 1)
        s.step(1)
    s.synchronize()
    x = s.positions()
    assert np.isfinite(x).all()
    np.testing.assert_allclose(x[w.fixed], w.X[w.fixed], atol=1e-7)  # float32 storage of the rest state
    np.testing.assert_allclose(x[w.kin_idx], w.X[w.kin_idx] + w.kin_offset(3), atol=1e-6)
    h = s.residual_history()
    assert h.shape == (w.iters + 1,) and np.all(np.isfinite(h)) and h[-1] < h[0]
    nonfinite, _ = s.health()
    assert nonfinite == 0
    s.close()


def test_beam_full_size_with_sphere(lib):
    w = W.beam()
    s = W.make_solver(w)
    seen = 0
    for k in range(40):
        W.drive_gpu(s, w, k)
        s.step(1)
        if k in (11, 21, 31):
            seen += len(s.collisions())
    x = s.positions()
    assert seen > 0
    assert np.isfinite(x).all()
    np.testing.assert_allclose(x[w.fixed], w.X[w.fixed], atol=1e-7)
    s.close()


def test_residual_history_follows_set_num_iters(lib):
    X, tets, faces, x0 = _noisy_cube(3, seed=8)
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, num_iters=4, residual_policy=G.RESIDUAL_EVERY_ITERATION)
    s.set_positions(x0)
    s.step(1)
    assert len(s.residual_history()) == 5
    s.set_num_iters(40)
    s.step(1)
    h = s.residual_history()
    assert len(h) == 41 and np.all(np.isfinite(h)) and h[-1] < h[0]
    s.close()


def _flow_case():
    X, tets, _ = G.grid_mesh(9, 7, 8, 0.02)
    T = tets.shape[0]
    E = np.exp(np.random.default_rng(3).uniform(np.log(1e3), np.log(1e5), T))
    x0 = X + np.random.default_rng(4).uniform(-5e-4, 5e-4, X.shape)
    return X, tets, E, x0


def _run_flow_case(var, iters, steps, policy=G.RESIDUAL_NEVER):
    X, tets, E, x0 = _flow_case()
    s = G.XPBDSolver(X, tets, None, E, 0.45, 1000.0, num_iters=iters, gs_variant=var, residual_policy=policy)
    s.fix_vertices(X[:, 2] == 0)
    s.set_positions(x0)
    s.step(steps)
    out = (s.positions(), s.lambdas(), s.residual_history() if policy != G.RESIDUAL_NEVER else None)
    s.synchronize()
    s.close()
    return out


def test_dataflow_single_sweep_matches_launch_order(lib):
    """One sweep from a perturbed state: the dataflow sweep and the colour
    launches differ by FP32 rounding at most (an ordering error would show as
    a whole Gauss-Seidel update, ~1e-5 m here)."""
    a = _run_flow_case(0, 1, 1)[0]
    for var in (1, 2, 3, 4):
        b = _run_flow_case(var, 1, 1)[0]
        assert np.abs(a - b).max() <= 4e-8, (var, np.abs(a - b).max())


@pytest.mark.parametrize("var", [2, 3, 4])
@pytest.mark.parametrize("policy", [G.RESIDUAL_NEVER, G.RESIDUAL_EVERY_SUBSTEP, G.RESIDUAL_EVERY_ITERATION])
def test_dataflow_sweep_is_deterministic_and_close(lib, policy, var):
    """Sweep variants 2 and 3 (one cooperative launch, per-task dependency
    counters; 3 with bulk-copied records) project the same patches in the
    same order as the colour-by-colour launches of variants 0 and 1, and
    variant 4 (vertex versions) in the same order as variant 2: results do
    not depend on timing (bit-identical reruns) and stay within FP32
    rounding drift of the reference variant after 25 steps x 12 iterations;
    with the per-iteration residual they run the colour launches themselves."""
    r0 = _run_flow_case(var, 12, 25, policy)
    r1 = _run_flow_case(var, 12, 25, policy)
    ref = _run_flow_case(var - 2, 12, 25, policy)
    np.testing.assert_array_equal(r0[0], r1[0])
    np.testing.assert_array_equal(r0[1], r1[1])
    assert np.abs(r0[0] - ref[0]).max() <= 2e-6
    if policy == G.RESIDUAL_EVERY_ITERATION:
        np.testing.assert_array_equal(r0[0], ref[0])
    if policy != G.RESIDUAL_NEVER:
        # the final residual sits near the FP32 floor (~1e-7 of the first)
        np.testing.assert_allclose(r0[2], ref[2], rtol=1e-3, atol=1e-6 * ref[2][0])


@pytest.mark.parametrize("var", [2, 3, 4])
def test_dataflow_sweep_full_block(lib, var):
    """The 1.31M-tet block, one kinematically driven step: variant 2 is
    reproducible bit for bit and within FP32 rounding of variant 0. (Over
    several steps rounding-level differences between any two sweep kernels
    grow on this stiff, unconverged block: variants 0 and 1 differ by 2e-4 m
    after three steps, as do 0 and 2.)"""
    w = W.block()
    out = []
    for v in (var, 0, var):
        s = W.make_solver(w, gs_variant=v)
        W.drive_gpu(s, w, 1)
        s.step(1)
        s.synchronize()
        out.append(s.positions())
        nonfinite, _ = s.health()
        assert nonfinite == 0
        s.close()
    np.testing.assert_array_equal(out[0], out[2])
    assert np.abs(out[0] - out[1]).max() <= 1e-6


def test_versioned_sweep_equals_fenced_sweep_over_100_block_steps(lib):
    """Variant 4 reads a vertex as four 64-bit words, each coordinate beside
    the version it was written with, and polls again unless all three carry
    the due version; variant 2 orders the same sweep with release/acquire
    alone. On the 1.31M-tet block driven for 100 substeps (3,000 sweeps,
    1,024 warps racing on shared vertices), two variant-4 runs and a
    variant-2 run end bit-identical."""
    w = W.block()
    out = []
    for var in (4, 4, 2):
        s = W.make_solver(w, gs_variant=var)
        for k in range(100):
            W.drive_gpu(s, w, k + 1)
            s.step(1)
        s.synchronize()
        assert s.health()[0] == 0
        out.append(s.positions())
        s.close()
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[0], out[2])


def _fan(n=300, seed=7):
    """n tets that share vertex 0 and nothing else, so every tet is its own
    colour and vertex 0 lies in n single-tet patches."""
    rng = np.random.default_rng(seed)
    X, tets = [np.zeros(3)], []
    for _ in range(n):
        d = rng.normal(size=3)
        c = 0.05 * d / np.linalg.norm(d)
        base = len(X)
        X.extend(c + 0.02 * rng.normal(size=(3, 3)))
        tets.append([0, base, base + 1, base + 2])
    return np.array(X), np.array(tets, dtype=np.int32)


def _launches_and_positions(X, tets, var, steps=2, **kw):
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, num_iters=4, gs_variant=var, **kw)
    s.step(1)
    s.synchronize()
    l0 = s.launch_count()
    s.step(steps)
    s.synchronize()
    n, x = s.launch_count() - l0, s.positions()
    s.close()
    return n, x


def test_versioned_sweep_falls_back_past_255_patches_per_vertex(lib):
    """Variant 4 keeps deg and pre of a vertex in 8 bits each. A vertex in more
    than 255 patches makes the context run the task-counter sweep (variant 2)
    instead of failing: the same launches and bit-identical positions as
    variant 2, the colour launches' order. On a regular mesh variant 4 runs its
    own sweep: two more launches per step (the version copies in and out)."""
    X, tets = _fan()
    n4, x4 = _launches_and_positions(X, tets, 4, gs_patch_tets=1)
    n2, x2 = _launches_and_positions(X, tets, 2, gs_patch_tets=1)
    _, x0 = _launches_and_positions(X, tets, 0, gs_patch_tets=1)
    assert n4 == n2
    np.testing.assert_array_equal(x4, x2)
    assert np.abs(x2 - x0).max() <= 1e-6
    w = W.cube(n=4)
    m4, _ = _launches_and_positions(w.X, w.tets, 4)
    m2, _ = _launches_and_positions(w.X, w.tets, 2)
    assert m4 == m2 + 2 * 2


@pytest.mark.parametrize("solver,adjust", [(G.SOLVER_GAUSS_SEIDEL, 0), (G.SOLVER_JACOBI, 0),
                                           (G.SOLVER_GAUSS_SEIDEL, 1)])
def test_first_order_trajectory_matches_fp64_oracle(lib, solver, adjust):
    """FirstOrderXPBDMeshObject: alpha~ = alpha/dt, vertex damping as the
    constraint inertia, gravity as -g m dt / B per step; bottom fixed, 60
    steps against the FP64 oracle (GPU sweep order replayed)."""
    X, tets, faces, x0 = _noisy_cube(5, seed=11)
    mult = 2e4 if not adjust else 2.0
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, num_iters=8, solver_type=solver, first_order=1,
                     damping_multiplier=mult, adjust_damping_to_material=adjust)
    o32, o64 = _oracle_pair(X, tets, faces, 3e3, 0.45, 1000.0, solver, 8, gpu=s)
    fixed = X[:, 2] == 0
    s.set_positions(x0); s.fix_vertices(fixed)
    for o in (o32, o64):
        o.set_first_order(mult, adjust=bool(adjust))
        o.set_positions(x0); o.set_fixed(fixed)
    s.step(60); o32.time_steps(60); o64.time_steps(60)
    band = np.abs(o32.positions() - o64.positions()).max()
    err = np.abs(s.positions() - o64.positions()).max()
    assert err <= max(1e-4 * _extent(X), 3 * band), (err, band)
    # the body moved (gravity acts through the damping)
    assert np.abs(s.positions() - x0).max() > 1e-4
    s.close()


@pytest.mark.parametrize("solver", [G.SOLVER_GAUSS_SEIDEL, G.SOLVER_JACOBI])
def test_attachments_match_fp32_oracle(lib, solver):
    """Grasping-style attachments: two top vertices attached (one through an
    offset) to points that rise 0.1 mm per step; bottom fixed; 15 steps.
    Compared with the FP32 oracle: below |x - target| = 1e-12 the reference's
    gradient falls back to (1e-12, 1e-12, 1e-12), which turns a rounding-level
    distance into a jump of -C / 3e-12 per coordinate. FP64 runs reach that
    branch after a vertex has been snapped onto its target (distances of
    1e-13 .. 1e-15); FP32 distances between coordinates away from 0 never fall
    below it except at exactly 0, where the update is 0 -- so the FP64
    trajectory is not a usable reference here."""
    X, tets, faces, x0 = _noisy_cube(4, seed=21, noise=1e-3)
    s = G.XPBDSolver(X, tets, None, 3e4, 0.4, 1000.0, num_iters=8, solver_type=solver)
    o = O.Oracle(X, tets, faces, 3e4, 0.4, 1000.0, num_iter=8, precision=32,
                 solver=O.JACOBI if solver == G.SOLVER_JACOBI else O.COLOURED_GS)
    if solver == G.SOLVER_GAUSS_SEIDEL:
        o.set_order(s.sweep_order())
    fixed = X[:, 2] == 0
    s.set_positions(x0); s.fix_vertices(fixed)
    o.set_positions(x0); o.set_fixed(fixed)
    # top vertices away from the coordinate planes (no sub-1e-12 float spacing)
    top = np.nonzero((X[:, 2] == X[:, 2].max()) & (X[:, 0] >= 0.25) & (X[:, 1] >= 0.25))[0]
    v1, v2 = int(top[0]), int(top[-1])
    off = np.array([0.0, 0.0, 0.002])
    a1 = s.add_attachment(v1, X[v1])
    a2 = s.add_attachment(v2, X[v2] - off, off)
    o.add_attachment(v1, X[v1])
    o.add_attachment(v2, X[v2])
    for k in range(15):
        lift = np.array([0, 0, 1e-4 * (k + 1)])
        s.set_attachment_point(a1, X[v1] + lift)
        s.set_attachment_point(a2, X[v2] - off + lift)
        o.set_attachment_target(0, X[v1] + lift)
        o.set_attachment_target(1, X[v2] + lift)
        s.update(); s.velocity_update()
        o.update(); o.velocity_update()
    err = np.abs(s.positions() - o.positions()).max()
    assert err <= 1e-5 * _extent(X), err
    # the attached vertex ends on its point (within Jacobi's summed updates)
    np.testing.assert_allclose(s.positions()[v1], X[v1] + [0, 0, 1.5e-3], atol=1e-6)
    s.close()
    o.close()
