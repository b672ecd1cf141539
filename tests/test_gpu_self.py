"""Self-collisions on the GPU (the grid query replacing Embree, the closest
rest-surface face, DeformableDeformableCollisionConstraint) against the
oracle: the same contacts from the same positions, and trajectories within
the FP32/FP64 band. Reference: XPBDMeshObject.cpp:719-762,
EmbreeScene.cpp:369-393, EmbreeTetMeshGeometry.cpp:20-47,
DeformableMeshSDF.cpp:68-82, DeformableDeformableCollisionConstraint.cpp."""
import numpy as np
import pytest

import oracle as O
import simulation as S
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def two_cubes(n=3, gap=0.005, shift=(0.0, 0.01, 0.005)):
    Xa, ta, fa = G.grid_mesh(n, n, n, 0.1 / n)
    Xb = Xa + np.array([0.1 + gap, shift[1], shift[2]])
    return np.vstack([Xa, Xb]), np.vstack([ta, ta + len(Xa)]), np.vstack([fa, fa + len(Xa)]), len(Xa)


@pytest.mark.parametrize("n,push", [(3, 0.008), (4, 0.012), (6, 0.02)])
def test_detection_matches_oracle(lib, n, push):
    """One cube pushed into the other: the GPU finds the same (vertex, face)
    pairs, in the same order, as the oracle's brute-force restatement of the
    Embree queries (positions given in float, so both test the same values)."""
    X, tets, faces, na = two_cubes(n=n, gap=0.002, shift=(0, 0.013, 0.007))
    x = X.copy()
    x[:na, 0] += push
    x[:na, 2] += 0.003 * np.sin(40 * x[:na, 1])
    x = x.astype(np.float32).astype(np.float64)
    s = G.XPBDSolver(X, tets, faces, 3e3, 0.45, 1000.0, g_accel=0.0, self_collisions=1)
    o = O.Oracle(X, tets, faces, 3e3, 0.45, 1000.0, g=0.0, precision=32)
    o.enable_self_collisions()
    s.set_positions(x)
    o.set_positions(x)
    s.detect_collisions()
    o.detect()
    vf, _ = s.self_contacts()
    exp = o.self_contacts()[:, :2].astype(np.int32)
    assert len(exp) >= 4
    np.testing.assert_array_equal(vf, exp)
    s.close(); o.close()


@pytest.mark.parametrize("solver", [G.SOLVER_GAUSS_SEIDEL, G.SOLVER_JACOBI])
def test_colliding_cubes_match_oracle(lib, solver):
    """Two cubes of one mesh meeting at 1 m/s, self-collision detection every
    step: positions against the FP64 oracle within max(1e-4 x extent, 3 x the
    FP32/FP64 oracle band), and the cubes stopped."""
    X, tets, faces, na = two_cubes()
    v = np.zeros_like(X)
    v[:na, 0], v[na:, 0] = 1.0, -1.0
    s = G.XPBDSolver(X, tets, faces, 2e4, 0.45, 1000.0, g_accel=0.0, num_iters=8, solver_type=solver,
                     collision_rate=1000.0, self_collisions=1)
    os_ = [O.Oracle(X, tets, faces, 2e4, 0.45, 1000.0, g=0.0, num_iter=8, precision=prec,
                    solver=O.JACOBI if solver == G.SOLVER_JACOBI else O.COLOURED_GS) for prec in (32, 64)]
    s.set_velocities(v)
    for o in os_:
        if solver == G.SOLVER_GAUSS_SEIDEL:
            o.set_order(s.sweep_order())
        o.set_collision_rate(1000.0)
        o.enable_self_collisions()
        o.set_velocities(v)
    for _ in range(20):
        s.step(1)
        for o in os_:
            o.time_steps(1)
    assert s.health()[0] == 0
    band = np.abs(os_[0].positions() - os_[1].positions()).max()
    err = np.abs(s.positions() - os_[1].positions()).max()
    assert err <= max(1e-4 * 0.2, 3 * band), (err, band)
    x = s.positions()
    assert x[:na, 0].max() - x[na:, 0].min() < 0.1 / 3 * 0.5
    s.close()


SCENE = """
name: "Fold"
visualization: "None"
sim-mode: "AFAP"
time-step: 1e-3
collision-rate: 1000
end-time: 0.02
g-accel: 0
materials:
  - name: "Tissue"
    density: 1000
    E: 2e4
    nu: 0.45
objects:
  - name: "Pair"
    type: "XPBDMeshObject"
    filename: "pair.msh"
    materials: ["Tissue"]
    collisions: true
    self-collisions: true
    num-solver-iters: 8
    solver-type: "Gauss-Seidel"
"""


def test_self_collisions_from_config(lib, tmp_path):
    """self-collisions: true in a YAML scene equals the hand-driven solver."""
    import msh
    X, tets, faces, na = two_cubes()
    msh.write_msh(str(tmp_path / "pair.msh"), X, tets, faces)
    with S.Simulation(SCENE, base_dir=str(tmp_path)) as sim:
        sim.setup()
        sim.objects["Pair"].solver.set_velocities(np.where(np.arange(len(X))[:, None] < na, 1.0, -1.0) *
                                                  np.array([1.0, 0, 0]))
        steps = sim.update()
        got = sim.objects["Pair"].positions()
    Xp = msh.place(X, faces, (0, 0, 0), (0, 0, 0), None, None)
    s = G.XPBDSolver(Xp, tets, faces, 2e4, 0.45, 1000.0, g_accel=0.0, num_iters=8, collision_rate=1000.0,
                     self_collisions=1)
    s.set_velocities(np.where(np.arange(len(X))[:, None] < na, 1.0, -1.0) * np.array([1.0, 0, 0]))
    s.step(steps)
    np.testing.assert_array_equal(got, s.positions())
    assert len(s.self_contacts()[0]) > 0
    s.close()
