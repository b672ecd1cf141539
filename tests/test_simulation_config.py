"""CPU checks of the configuration layer: the YAML subset reader, the config
defaults of the reference's config classes, the gmsh reader/writer and the
mesh placement (MeshObject::loadAndConfigureMesh)."""
import os

import numpy as np
import pytest

import msh
import simulation as S
import xpbd_gb300 as G
import yaml_lite as Y
from conftest import reference_dir

REF = reference_dir()
REF_CONFIGS = os.path.join(REF, "config") if REF else None

CONFIG = """
## a test scene
name: "Scene"   # name
description: 'two objects'
visualization: "None"
g-accel: 9.81
sim-mode: "AFAP"
time-step: 1e-3
collision-rate: 100
end-time: 0.05

materials:
  -
    name: "Soft"
    density: 1000
    E: 3e3
    nu: 0.45
  - name: "Stiff"
    E: 3e4

objects:
  -
    name: "Cube"
    type: "XPBDMeshObject"
    filename: "cube.msh"
    materials: ["Soft", "Stiff"]
    max-size: 1
    position: [0, 0, 0.5]
    velocity: [0, 0, 0]
    rotation: [0, 0, 30]
    collisions: true
    num-solver-iters: 5
    solver-type: "Gauss-Seidel"
    constraint-type: "Stable-Neohookean-Combined"
    residual-policy: "Never"
    colors: [
      [1, 0, 0],
      [0, 1, 0]
    ]
  - name: "Ball"
    type: "RigidSphere"
    radius: 0.2
    position: [0, 0, 1.15]
    fixed: true
    collisions: true
"""


def test_yaml_subset():
    d = Y.loads(CONFIG)
    assert d["name"] == "Scene" and d["description"] == "two objects"
    assert d["time-step"] == 1e-3 and isinstance(d["collision-rate"], int)
    assert d["materials"][1] == {"name": "Stiff", "E": 3e4}
    cube = d["objects"][0]
    assert cube["materials"] == ["Soft", "Stiff"] and cube["position"] == [0, 0, 0.5]
    assert cube["colors"] == [[1, 0, 0], [0, 1, 0]] and cube["collisions"] is True
    assert Y.scalar("~") is None and Y.scalar("off") is False and Y.scalar(".5") == 0.5
    with pytest.raises(ValueError):
        Y.loads("a: &anchor 1")


@pytest.mark.skipif(not (REF_CONFIGS and os.path.isdir(REF_CONFIGS)), reason="reference configs not present")
def test_every_reference_config_parses():
    import glob
    files = sorted(glob.glob(os.path.join(REF_CONFIGS, "**", "*.yaml"), recursive=True))
    assert files
    for f in files:
        d = Y.load(f)
        assert isinstance(d, dict) and "objects" in d, f


def test_config_defaults_follow_the_reference():
    c = S.SimulationConfig.from_node({})
    assert (c.time_step, c.end_time, c.g_accel, c.collision_rate, c.fps) == (1e-3, 10.0, 9.81, 100.0, 30.0)
    assert c.sim_mode == "Visualization" and c.visualization == "VTK"
    m = S.ElasticMaterialConfig.from_node({})
    assert (m.density, m.E, m.nu, m.mu_s, m.mu_k) == (1000.0, 3e6, 0.499, 0.5, 0.2)
    o = S.XPBDMeshObjectConfig.from_node({"name": "x"})
    assert o.num_solver_iters == 1 and o.num_local_collision_iters == 0 and not o.collisions
    assert o.solver_type == G.SOLVER_GAUSS_SEIDEL and o.constraint_type == G.CONSTRAINT_COMBINED
    assert o.residual_policy == G.RESIDUAL_NEVER and o.max_size is None and o.size is None
    s = S.RigidSphereConfig.from_node({})
    assert s.radius == 1.0 and s.fixed is False


def test_config_objects_and_errors():
    c, _ = S.load_config(CONFIG)
    assert [type(o).__name__ for o in c.objects] == ["XPBDMeshObjectConfig", "RigidSphereConfig"]
    cube = c.objects[0]
    assert cube.max_size == 1.0 and np.allclose(cube.rotation, [0, 0, 30]) and cube.num_solver_iters == 5
    assert c.materials[1].density == 1000.0 and c.materials[1].nu == 0.499
    with pytest.raises(ValueError):
        S.SimulationConfig.from_node({"objects": [{"type": "Teapot"}]})
    with pytest.raises(NotImplementedError):
        S.SimulationConfig.from_node({"objects": [{"type": "RigidMeshObject"}]})
    boxes = S.SimulationConfig.from_node({"objects": [{"type": "RigidBox", "size": [1, 2, 3], "fixed": True},
                                                      {"type": "RigidCylinder", "radius": 0.5}]})
    assert np.allclose(boxes.objects[0].size, [1, 2, 3]) and boxes.objects[0].fixed
    assert boxes.objects[1].radius == 0.5 and boxes.objects[1].height == 1.0
    fo = S.SimulationConfig.from_node({"objects": [{"type": "FirstOrderXPBDMeshObject", "damping-multiplier": 5e4}]})
    assert fo.objects[0].first_order and fo.objects[0].damping_multiplier == 5e4
    assert not fo.objects[0].adjust_damping_to_material
    with pytest.raises(ValueError):
        S.XPBDMeshObjectConfig.from_node({"solver-type": "Conjugate"})


def test_msh_round_trip(tmp_path):
    X, tets, faces = G.grid_mesh(3, 4, 2, 0.1)
    p = str(tmp_path / "m.msh")
    msh.write_msh(p, X, tets, faces)
    Y2, t2, f2 = msh.read_msh(p)
    np.testing.assert_array_equal(Y2, X)
    np.testing.assert_array_equal(t2, tets)
    np.testing.assert_array_equal(f2, faces)


def test_msh_reader_matches_reference_meshes():
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_meshes.npz"))
    for name in ("cube2", "cube4"):
        p = os.path.join(REF, "resource", "cube", f"{name}.msh") if REF else ""
        if not os.path.exists(p):
            pytest.skip("reference meshes not present")
        X, tets, faces = msh.read_msh(p)
        np.testing.assert_array_equal(X, g[f"{name}_X"])
        np.testing.assert_array_equal(tets, g[f"{name}_tets"])
        np.testing.assert_array_equal(faces, g[f"{name}_faces"])


def test_placement():
    X, tets, faces = G.grid_mesh(2, 2, 2, 0.5)  # unit cube at the origin corner
    # max-size scales about the origin, the surface centre of mass goes to position
    Y2 = msh.place(X, faces, position=(1, 2, 3), max_size=2.0)
    np.testing.assert_allclose(Y2.max(0) - Y2.min(0), [2, 2, 2])
    np.testing.assert_allclose(msh.mass_center(Y2, faces), [1, 2, 3], atol=1e-12)
    # per-axis size, then a rotation about position keeps the centre
    Y3 = msh.place(X, faces, position=(0, 0, 1), size=(1, 2, 4), rotation=(0, 0, 90))
    np.testing.assert_allclose(Y3.max(0) - Y3.min(0), [2, 1, 4], atol=1e-12)
    R = msh.rotation_xyz([10, 20, 30])
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
    assert np.isclose(np.linalg.det(R), 1.0)
    # x first, then y, then z: R = Rz Ry Rx
    def rx(a): return np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    def ry(a): return np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    def rz(a): return np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    d = np.radians([10, 20, 30])
    np.testing.assert_allclose(R, rz(d[2]) @ ry(d[1]) @ rx(d[0]), atol=1e-12)


def test_element_classes_file(tmp_path):
    p = tmp_path / "classes.txt"
    p.write_text("0\n1\n1\n0\nend\n2\n")
    np.testing.assert_array_equal(S.read_element_classes(str(p)), [0, 1, 1, 0])


def test_euler_quaternion_matches_the_rotation_matrix():
    for deg in ([0, 0, 0], [30, 0, 0], [10, 20, 30], [-45, 60, 170]):
        x, y, z, w = S.eul_xyz_to_quat(deg)
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        np.testing.assert_allclose(R, msh.rotation_xyz(deg), atol=1e-12)
