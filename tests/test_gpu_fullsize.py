"""Full-size parity on the benchmarked configurations, through the C ABI.

Block (1,310,720 tets, 274,625 vertices, per-tet E log-uniform [1e3, 1e5],
nu 0.45, bottom fixed, top face driven up, 30 coloured Gauss-Seidel sweeps):
the production sweep (the versioned one-launch kernel) against the FP64 and
FP32 oracles replaying the device's sweep order (xpbd_get_sweep_order), three
driven substeps. This solve is rounding-sensitive: from lambda = 0 the first
sweeps move vertices by millimetres before the large rest multipliers build
up, and velocities (x - prev) / dt carry an unconverged substep's rounding
into the next. Perturbing the FP64 oracle's start by 1e-12 m moves its
one-sweep state by 7 mm; the FP32 oracle -- an exact FP32 restatement of the
same arithmetic -- departs from the FP64 oracle by 0.2-0.6 mm in position and
by up to 60 % in a substep's final relative residual. So the bounds are the
FP32 band: max vertex error <= max(1e-4 x extent, 3 x band32), band32 =
|FP32 oracle - FP64 oracle|, and each substep's final relative residual
(FP64 evaluation, XPBDSolver.hpp:327-391) within a factor 2 of the FP64
oracle's. The benchmark's claim is checked directly as well: at its sweep
count to 1e-3 (88) every driven substep of the device and of the FP64 oracle
ends at a relative residual <= 1e-3, and the device first reaches 1e-3
within 15 % of that count of the FP32 oracle (FP64 arithmetic itself gets
there sooner after an unconverged substep: 64 against 86 sweeps in the
second).

Beam as specified (50,000 tets, 12,221 vertices, E 1e4, nu 0.49, y-min end
clamped, FP32 Jacobi with 20 sweeps, sphere r 0.03 m descending 0.05 m/s,
collision-rate 100 Hz). The reference's plain-sum Jacobi (XPBDJacobiSolver.hpp:79-114)
is unstable on this nearly incompressible beam: rounding is amplified every
sweep, so from the exact rest state the FP64 oracle moves 1e-5 m in the first
substep while the FP32 oracle moves 8 mm. Two checks:
  * kernels at full size: one substep with contacts detected at the start
    and 1, 2 or 4 sweeps (little amplification yet): device within
    max(1e-4 x extent, 3 x band32) of the FP64 oracle;
  * the run as specified, the device's detections fed to the oracles: every
    substep until the FP64 oracle has diverged the device stays within
    4 x band32 of it (both are amplified rounding, seeded differently), and
    the device and both oracles all move a vertex by more than the beam's
    length within 40 substeps.
"""
import numpy as np
import pytest

import oracle as O
import workloads as W
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _extent(X):
    return float((X.max(0) - X.min(0)).max())


def test_block_full_size_matches_fp64_and_fp32_oracles(lib):
    w = W.block()
    steps = 3
    s = W.make_solver(w)  # production: versioned one-launch sweep
    sr = W.make_solver(w, residual_policy=G.RESIDUAL_EVERY_ITERATION)  # colour launches, same order
    order = s.sweep_order()
    np.testing.assert_array_equal(order, sr.sweep_order())
    ors = []
    for prec in (64, 32):
        o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=w.iters,
                     solver=O.COLOURED_GS, precision=prec)
        o.set_order(order)
        o.set_fixed(w.fixed)
        o.set_kinematic_group(w.kin_idx)
        ors.append(o)
    o64, o32 = ors
    hists = []
    for k in range(1, steps + 1):
        off = w.kin_offset(k)
        for solver in (s, sr):
            solver.set_kinematic_offset(off)
            solver.step(1)
        for o in ors:
            o.set_kinematic_offset(off)
        o64.time_steps(1, record=True)
        o32.time_steps(1, record=True)
        h_gpu, h_ref, h32 = sr.residual_history(), o64.res_history(), o32.res_history()
        print(f"substep {k}: rel. residual history gpu {np.round(h_gpu[[1, 2, 5, 10, 30]] / h_gpu[0], 5)} "
              f"fp64 {np.round(h_ref[[1, 2, 5, 10, 30]] / h_ref[0], 5)} fp32 {np.round(h32[[1, 2, 5, 10, 30]] / h32[0], 5)}")
        hists.append((h_gpu, h_ref, h32))
    s.synchronize()
    assert s.health()[0] == 0
    band = np.abs(o32.positions() - o64.positions()).max()
    err = np.abs(s.positions() - o64.positions()).max()
    err_r = np.abs(sr.positions() - o64.positions()).max()
    bound = max(1e-4 * _extent(w.X), 3 * band)
    print(f"block, {steps} substeps: |gpu - fp64| {err:.3e} (colour launches {err_r:.3e}), band32 {band:.3e}, "
          f"bound {bound:.3e}, |gpu - fp32| {np.abs(s.positions() - o32.positions()).max():.3e}")
    # substep 1 starts from the same predicted state: r(x_pred, 0) agrees
    assert abs(hists[0][0][0] / hists[0][1][0] - 1) <= 1e-6
    for h_gpu, h_ref, h32 in hists:
        assert h_gpu.shape == h_ref.shape == (w.iters + 1,)
        rg, r64, r32 = (h[-1] / h[0] for h in (h_gpu, h_ref, h32))
        assert 0.5 <= rg / r64 <= 2.0, (rg, r64, r32)
    assert err <= bound and err_r <= bound
    np.testing.assert_allclose(s.positions()[w.kin_idx], w.X[w.kin_idx] + w.kin_offset(steps), atol=1e-6)
    for o in ors:
        o.close()
    s.close()
    sr.close()


def test_block_reaches_1e3_in_88_sweeps_in_fp32_and_fp64(lib):
    w = W.block()
    sweeps = 88  # the benchmark's calibrated count (most over 24 driven substeps)
    s = W.make_solver(w, residual_policy=G.RESIDUAL_EVERY_ITERATION, num_iters=sweeps)
    ors = []
    for prec in (64, 32):
        o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=sweeps, solver=O.COLOURED_GS,
                     precision=prec)
        o.set_order(s.sweep_order())
        o.set_fixed(w.fixed)
        o.set_kinematic_group(w.kin_idx)
        ors.append(o)
    for k in range(1, 4):
        off = w.kin_offset(k)
        s.set_kinematic_offset(off)
        s.step(1)
        for o in ors:
            o.set_kinematic_offset(off)
            o.time_steps(1, record=True)
        rg, r64, r32 = (h / h[0] for h in (s.residual_history(), ors[0].res_history(), ors[1].res_history()))
        fg, f64, f32 = (int(np.argmax(r <= 1e-3)) for r in (rg, r64, r32))
        print(f"block, substep {k}, {sweeps} sweeps: final rel. residual gpu {rg[-1]:.3e} fp64 {r64[-1]:.3e} "
              f"fp32 {r32[-1]:.3e}; first sweep at 1e-3 gpu {fg} fp64 {f64} fp32 {f32}")
        # the count holds in FP64 too, and the device converges as FP32 arithmetic does
        assert rg[-1] <= 1e-3 and r64[-1] <= 1e-3
        assert abs(fg - f32) <= 0.15 * sweeps
    for o in ors:
        o.close()
    s.close()


def _beam_pair_oracles(w, iters):
    ors = []
    for prec in (64, 32):
        o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=iters, solver=O.JACOBI,
                     precision=prec)
        o.set_fixed(w.fixed)
        ors.append(o)
    return ors


@pytest.mark.parametrize("iters", [1, 2, 4])
def test_beam_as_specified_one_substep_with_contacts(lib, iters):
    w = W.beam(jacobi=True)
    assert (w.T, w.V, w.iters) == (50_000, 12_221, 20)
    s = W.make_solver(w, num_iters=iters)
    o64, o32 = _beam_pair_oracles(w, iters)
    s.set_spheres(w.sphere_centre(0.0), [w.sphere_r])
    s.detect_collisions()
    rows = s.collisions()
    assert len(rows) > 0
    for o in (o64, o32):
        o.set_contacts(rows)
        o.update()
    s.update()
    band = np.abs(o32.positions() - o64.positions()).max()
    err = np.abs(s.positions() - o64.positions()).max()
    moved = np.abs(o64.positions() - w.X).max()
    print(f"beam, {iters} sweeps, {len(rows)} contacts: moved {moved:.3e}, |gpu - fp64| {err:.3e}, band32 {band:.3e}")
    assert moved > 1e-5
    assert err <= max(1e-4 * _extent(w.X), 3 * band)
    for o in (o64, o32):
        o.close()
    s.close()


def test_beam_as_specified_jacobi_diverges_in_both(lib):
    w = W.beam(jacobi=True)
    s = W.make_solver(w)
    o64, o32 = _beam_pair_oracles(w, w.iters)
    ors = (o64, o32)
    length = _extent(w.X)
    floor = 1e-4 * length
    t, last, interval = 0.0, 0.0, 1.0 / w.collision_rate
    div = {"gpu": None, "fp64": None, "fp32": None}
    ncontacts = 0
    worst = 0.0
    for k in range(1, 41):
        if t - last > interval:
            s.set_spheres(w.sphere_centre(t), [w.sphere_r])
            s.detect_collisions()
            rows = s.collisions()
            ncontacts += len(rows)
            for o in ors:
                o.set_contacts(rows)
        s.update()
        s.velocity_update()
        for o in ors:
            o.update()
            o.velocity_update()
        if t - last > interval:
            last = t
        t += w.dt
        xs, xo, x32 = s.positions(), o64.positions(), o32.positions()
        for name, x in (("gpu", xs), ("fp64", xo), ("fp32", x32)):
            dev = np.abs(x - w.X).max() if np.isfinite(x).all() else np.inf
            if div[name] is None and dev > length:
                div[name] = k
        if div["fp64"] is None:
            band = np.abs(x32 - xo).max()
            err = np.abs(xs - xo).max()
            worst = max(worst, err / max(floor, 4 * band))
            assert err <= max(floor, 4 * band), (k, err, band)
    print(f"beam Jacobi as specified: more than one beam length from rest at substep {div}; "
          f"{ncontacts} contacts injected; worst error / bound before the FP64 divergence {worst:.3f}")
    assert ncontacts > 0
    assert all(v is not None for v in div.values()), div
    for o in ors:
        o.close()
    s.close()
