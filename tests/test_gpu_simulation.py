"""The YAML-configured Simulation loop on the GPU: equal to driving the
solver by hand with the same placed mesh and parameters, and to the FP64
oracle."""
import numpy as np
import pytest

import msh
import oracle as O
import simulation as S
import xpbd_gb300 as G

pytestmark = pytest.mark.gpu

SCENE = """
name: "Scene"
visualization: "None"
sim-mode: "AFAP"
time-step: 1e-3
collision-rate: 100
end-time: {end}
g-accel: 9.81
materials:
  - name: "Soft"
    density: 1000
    E: 3e3
    nu: 0.45
  - name: "Stiff"
    density: 1200
    E: 3e4
    nu: 0.4
objects:
  - name: "Cube"
    type: "XPBDMeshObject"
    filename: "cube.msh"
    materials: ["Soft", "Stiff"]
    {classes}
    max-size: 0.5
    position: [0.1, 0, 0.5]
    rotation: [0, 0, 30]
    collisions: {coll}
    num-solver-iters: 6
    solver-type: "{solver}"
  - name: "Ball"
    type: "RigidSphere"
    radius: 0.2
    position: [0.1, 0, 0.93]
    fixed: true
    collisions: true
"""


def _scene(tmp_path, end=0.04, coll="true", solver="Gauss-Seidel", classes=None):
    X, tets, faces = G.grid_mesh(4, 4, 4, 0.25)
    msh.write_msh(str(tmp_path / "cube.msh"), X, tets, faces)
    cl = ""
    if classes is not None:
        (tmp_path / "classes.txt").write_text("\n".join(str(int(c)) for c in classes) + "\n")
        cl = 'element-classes-filename: "classes.txt"'
    cfg = tmp_path / "scene.yaml"
    cfg.write_text(SCENE.format(end=end, coll=coll, solver=solver, classes=cl))
    return str(cfg), X, tets, faces


def test_simulation_equals_the_solver_driven_by_hand(lib, tmp_path):
    """Gauss-Seidel is bit-reproducible, so the configured loop must equal the
    hand-driven solver exactly (the plain-sum Jacobi's float atomics are not)."""
    solver = "Gauss-Seidel"
    cfg, X, tets, faces = _scene(tmp_path, solver=solver)
    with S.Simulation(cfg) as sim:
        sim.setup()
        n = sim.update()
        assert n == 40 and abs(sim.time - 0.04) < 1e-12
        got = sim.objects["Cube"].positions()
    Xp = msh.place(X, faces, (0.1, 0, 0.5), (0, 0, 30), 0.5, None)
    T = tets.shape[0]
    s = G.XPBDSolver(Xp, tets, faces, np.full(T, 3e3), np.full(T, 0.45), np.full(T, 1000.0), dt=1e-3,
                     collision_rate=100, num_iters=6, solver_type=G.SOLVER_TYPES[solver])
    s.set_spheres([[0.1, 0, 0.93]], [0.2])
    s.step(40)
    np.testing.assert_array_equal(got, s.positions())
    # the sphere, 2 cm into the top face at the start, changed the motion
    free = G.XPBDSolver(Xp, tets, None, np.full(T, 3e3), np.full(T, 0.45), np.full(T, 1000.0), dt=1e-3,
                        num_iters=6)
    free.step(40)
    assert np.abs(free.positions() - got).max() > 1e-3
    s.close()
    free.close()


def test_element_classes_pick_materials(lib, tmp_path):
    X, tets, faces = G.grid_mesh(4, 4, 4, 0.25)
    classes = (np.arange(tets.shape[0]) % 3 == 0).astype(int)
    cfg, _, _, _ = _scene(tmp_path, coll="false", classes=classes)
    with S.Simulation(cfg) as sim:
        sim.setup()
        o = sim.objects["Cube"]
        np.testing.assert_array_equal(o.E, np.where(classes == 1, 3e4, 3e3))
        np.testing.assert_array_equal(o.rho, np.where(classes == 1, 1200.0, 1000.0))
        sim.update()
        got = o.positions()
    Xp = msh.place(X, faces, (0.1, 0, 0.5), (0, 0, 30), 0.5, None)
    ref = O.Oracle(Xp, tets, faces, np.where(classes == 1, 3e4, 3e3), np.where(classes == 1, 0.4, 0.45),
                   np.where(classes == 1, 1200.0, 1000.0), dt=1e-3, g=9.81, num_iter=6, solver=O.COLOURED_GS)
    order_solver = G.XPBDSolver(Xp, tets, None, 3e3, 0.45, 1000.0, num_iters=6)
    ref.set_order(order_solver.sweep_order())
    order_solver.close()
    ref.time_steps(40)
    err = np.abs(got - ref.positions()).max()
    assert err <= 1e-4 * 0.5, err
    ref.close()


def test_unprovided_objects_fail_loudly(lib, tmp_path):
    cfg, _, _, _ = _scene(tmp_path)
    text = open(cfg).read()
    # a free body colliding with two XPBD objects
    second = text[text.index('  - name: "Cube"'):text.index('  - name: "Ball"')].replace('"Cube"', '"Cube2"')
    two = text.replace("fixed: true", "fixed: false").replace('  - name: "Ball"', second + '  - name: "Ball"')
    with pytest.raises(NotImplementedError):
        S.Simulation(two, base_dir=str(tmp_path)).setup()


def test_first_order_object_from_config(lib, tmp_path):
    cfg, X, tets, faces = _scene(tmp_path, coll="false")
    text = open(cfg).read().replace('type: "XPBDMeshObject"',
                                    'type: "FirstOrderXPBDMeshObject"\n    damping-multiplier: 5e3')
    with S.Simulation(text, base_dir=str(tmp_path)) as sim:
        sim.setup()
        sim.update()
        got = sim.objects["Cube"].positions()
    Xp = msh.place(X, faces, (0.1, 0, 0.5), (0, 0, 30), 0.5, None)
    T = tets.shape[0]
    s = G.XPBDSolver(Xp, tets, None, np.full(T, 3e3), np.full(T, 0.45), np.full(T, 1000.0), dt=1e-3, num_iters=6,
                     first_order=1, damping_multiplier=5e3)
    s.step(40)
    np.testing.assert_array_equal(got, s.positions())
    # unconstrained 1st-order body: a rigid drift of -g rho dt / multiplier per step
    np.testing.assert_allclose(got - Xp, np.broadcast_to([0, 0, -40 * 9.81 * 1000 * 1e-3 / 5e3], Xp.shape),
                               atol=2e-6)
    s.close()


def test_fixed_box_and_cylinder_from_config(lib, tmp_path):
    """RigidBox / RigidCylinder objects become SDFs with the reference's
    orientation convention; the configured loop equals the hand-driven solver."""
    cfg, X, tets, faces = _scene(tmp_path)
    text = open(cfg).read().replace('''  - name: "Ball"
    type: "RigidSphere"
    radius: 0.2
    position: [0.1, 0, 0.93]''', '''  - name: "Slab"
    type: "RigidBox"
    size: [0.6, 0.6, 0.1]
    rotation: [0, 0, 20]
    position: [0.1, 0, 0.79]
    fixed: true
    collisions: true
  - name: "Post"
    type: "RigidCylinder"
    radius: 0.1
    height: 0.4
    rotation: [90, 0, 0]
    position: [0.1, 0, 0.2]''')
    with S.Simulation(text, base_dir=str(tmp_path)) as sim:
        sim.setup()
        assert set(sim.rigids) == {"Slab", "Post"}
        sim.update()
        got = sim.objects["Cube"].positions()
    Xp = msh.place(X, faces, (0.1, 0, 0.5), (0, 0, 30), 0.5, None)
    T = tets.shape[0]
    s = G.XPBDSolver(Xp, tets, faces, np.full(T, 3e3), np.full(T, 0.45), np.full(T, 1000.0), dt=1e-3,
                     collision_rate=100, num_iters=6)
    s.set_sdfs([G.SDF_BOX, G.SDF_CYLINDER], [[0.1, 0, 0.79], [0.1, 0, 0.2]],
               [S.rigid_quat([0, 0, 20]), S.rigid_quat([90, 0, 0])], [[0.6, 0.6, 0.1], [0.1, 0.4, 0]])
    s.step(40)
    np.testing.assert_array_equal(got, s.positions())
    s.close()
