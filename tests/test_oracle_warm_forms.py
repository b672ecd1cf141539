"""Warm starts of the multipliers, measured on the FP64 oracle (the learned
warm start's design question; the reference itself resets lambda at every
solve, XPBDSolver.hpp:71-77).

A driven block (per-tet E log-uniform [1e3, 1e5], top face raised, the
reference's sequential Gauss-Seidel) is followed along its converged
trajectory (every substep solved to 1e-9 relative residual). From each
converged state, one substep is solved by
  plain       lambda_0 = 0, x_0 = x_pred (the reference);
  lam_only    lambda_0 = the previous substep's lambda, x_0 = x_pred;
  disp_reuse  lambda_0 = the previous lambda, x_0 = x_pred + the previous
              substep's constraint correction (x_solved - x_pred);
each sweeping until ||r|| <= tol * ||r(x_pred, 0)|| (the plain normaliser),
and compared with that substep's converged solution. (The consistent form
the device uses, x_0 = x_pred + M^-1 grad C(x_pred)^T lambda_0, starts above
the plain residual: the rest multipliers are large, and so is the
linearisation error of their correction.) The two dual warm starts reach 1e-3
in fewer sweeps but land farther from the solution than the plain solver at
1e-3, with an error floor that a tighter tolerance does not lower -- the
start's force M^-1 grad C^T lambda_0 is missing (lam_only) or taken at the
old gradients (disp_reuse) -- and the plain solver at a looser tolerance
reaches their accuracy in fewer sweeps than they take. No form gains at
equal accuracy.
"""
import numpy as np
import pytest

import oracle as O
import workloads as W

N, K = 16, 6


def test_lambda_warm_starts_gain_nothing_at_equal_accuracy(oracle_mod):
    w = W.block(n=N, mesher=O.grid_mesh)
    o = O.Oracle(w.X, w.tets, w.faces, w.E, w.nu, w.rho, dt=w.dt, g=w.g, num_iter=600, solver=O.GAUSS_SEIDEL)
    o.set_fixed(w.fixed)
    o.set_kinematic_group(w.kin_idx)
    g = np.array([0.0, 0.0, -w.g * w.dt * w.dt])

    def step(x, v, k, mode, tol, lam_prev=None, dx_prev=None):
        o.set_positions(x)
        o.set_velocities(v)
        o.set_kinematic_offset(w.kin_offset(k))
        o.set_rel_tol(tol)
        if mode == "plain":
            o.update_start(None, None, record=True)
        elif mode == "lam_only":
            o.update_start(None, lam_prev, record=True)
        else:
            o.update_start(dx_prev, lam_prev, record=True)
        return o.positions(), o.iters_done(), o.lambdas(), o.res_history()[0] / o.last_r_plain()

    runs = [("plain", 1e-3), ("plain", 1e-2), ("lam_only", 1e-3), ("disp_reuse", 1e-3), ("lam_only", 1e-4)]
    sweeps = {r: 0 for r in runs}
    worst = {r: 0.0 for r in runs}
    start = {r: 0.0 for r in runs}
    x, v = w.X.copy(), np.zeros_like(w.X)
    lam_prev = dx_prev = None
    for k in range(1, K + 1):
        xs, _, lam, _ = step(x, v, k, "plain", 1e-9)
        if lam_prev is not None:
            for r in runs:
                xx, it, _, r0 = step(x, v, k, r[0], r[1], lam_prev, dx_prev)
                sweeps[r] += it
                worst[r] = max(worst[r], float(np.abs(xx - xs).max()))
                start[r] = max(start[r], r0)
        dx_prev, lam_prev = xs - (x + w.dt * v + g), lam
        v, x = (xs - x) / w.dt, xs
    o.close()
    print("per-substep solves from converged states: " +
          "; ".join(f"{m}@{t:g}: {sweeps[(m, t)]} sweeps, max error {worst[(m, t)]:.2e}" for m, t in runs))
    p3, p2, l3, d3, l4 = runs
    # the dual warm starts begin near the solution's residual and reach 1e-3 sooner ...
    assert start[l3] < 0.1 and start[d3] < 0.1
    assert sweeps[l3] < sweeps[p3] and sweeps[d3] < sweeps[p3]
    # ... but land farther from the solution, with a floor a tighter tolerance does not lower
    assert worst[l3] > 3 * worst[p3] and worst[d3] > 3 * worst[p3]
    assert worst[l4] > 0.8 * worst[l3]
    # the plain solver at a looser tolerance is as accurate for fewer sweeps
    assert sweeps[p2] < sweeps[l3] and worst[p2] < 2 * worst[l3]
