"""The reference's YAML-configured Simulation loop on the GB300 solver.

Configs (defaults as in the reference's config classes):
  SimulationConfig        include/config/simulation/SimulationConfig.hpp:75-138
  ElasticMaterialConfig   include/config/simobject/ElasticMaterialConfig.hpp:20-50
  ObjectConfig            include/config/simobject/ObjectConfig.hpp:28-62
  MeshObjectConfig        include/config/simobject/MeshObjectConfig.hpp:15-54
  XPBDMeshObjectConfig    include/config/simobject/XPBDMeshObjectConfig.hpp:62-125
  FirstOrderXPBDMeshObjectConfig  FirstOrderXPBDMeshObjectConfig.hpp:21-59
  RigidSphereConfig, RigidBoxConfig, RigidCylinderConfig
                          include/config/simobject/RigidPrimitiveConfigs.hpp:26-115,
                          RigidObjectConfig.hpp:18-41

Simulation mirrors src/simulation/Simulation.cpp:
  setup()      objects from their configs (Simulation.hpp:148-186): the mesh
               loaded from `filename` and placed (msh.place), materials by
               element class, the GPU solver with the object's solver keys
  update()     loop until end-time (Simulation.cpp:139-195); sim-mode
               "Visualization" keeps simulated time behind wall-clock time,
               "AFAP" and "Frame-by-frame" run free
  time_step()  _timeStep (Simulation.cpp:197-276): each object's xpbd_step
               runs collision detection on the shared cadence, the update and
               the velocity update

Fixed rigid spheres, boxes and cylinders with `collisions: true` collide with
every XPBD object that has `collisions: true`: each is a static SDF in the
solver (orientation from `rotation`, RigidObject.cpp:14) and can be moved
between steps (move_rigid). The reference only builds graphics for
`visualization`; there is no graphics here and the key is read and ignored.

Not provided (each raises NotImplementedError naming the key): non-fixed
rigid bodies (two-way coupling), rigid meshes, self-collisions and the
Virtuoso robot objects.
"""
from __future__ import annotations

import os
import time
from dataclasses import dataclass, field

import numpy as np

import msh
import xpbd_gb300 as G
import yaml_lite


def _get(node, key, default):
    v = node.get(key, default) if isinstance(node, dict) else default
    return default if v is None else v


def _vec3(node, key, default):
    v = _get(node, key, default)
    if not isinstance(v, (list, tuple)) or len(v) != 3:
        raise ValueError(f"{key}: expected a 3-vector, got {v!r}")
    return np.asarray(v, np.float64)


def _options(node, key, options, default):
    v = _get(node, key, default)
    if v not in options:
        raise ValueError(f"{key}: {v!r} is not one of {sorted(options)}")
    return options[v]


@dataclass
class ElasticMaterialConfig:
    name: str = ""
    density: float = 1000.0
    E: float = 3e6
    nu: float = 0.499
    mu_s: float = 0.5
    mu_k: float = 0.2

    @classmethod
    def from_node(cls, n):
        return cls(str(_get(n, "name", "")), float(_get(n, "density", 1000.0)), float(_get(n, "E", 3e6)),
                   float(_get(n, "nu", 0.499)), float(_get(n, "mu-s", 0.5)), float(_get(n, "mu-k", 0.2)))


SOLVER_TYPES = {"Gauss-Seidel": G.SOLVER_GAUSS_SEIDEL, "Jacobi": G.SOLVER_JACOBI,
                "Parallel-Jacobi": G.SOLVER_JACOBI}
CONSTRAINT_TYPES = {"Stable-Neohookean": G.CONSTRAINT_SEPARATE,
                    "Stable-Neohookean-Combined": G.CONSTRAINT_COMBINED}
RESIDUAL_POLICIES = {"Never": G.RESIDUAL_NEVER, "Every-Substep": G.RESIDUAL_EVERY_SUBSTEP,
                     "Every-Iteration": G.RESIDUAL_EVERY_ITERATION}


@dataclass
class XPBDMeshObjectConfig:
    name: str = ""
    collisions: bool = False
    graphics_only: bool = False
    position: np.ndarray = field(default_factory=lambda: np.zeros(3))
    velocity: np.ndarray = field(default_factory=lambda: np.zeros(3))
    rotation: np.ndarray = field(default_factory=lambda: np.zeros(3))
    filename: str = ""
    max_size: float | None = None
    size: np.ndarray | None = None
    materials: list = field(default_factory=list)
    element_classes_filename: str | None = None
    self_collisions: bool = False
    num_solver_iters: int = 1
    num_local_collision_iters: int = 0
    solver_type: int = G.SOLVER_GAUSS_SEIDEL
    constraint_type: int = G.CONSTRAINT_COMBINED
    residual_policy: int = G.RESIDUAL_NEVER
    first_order: bool = False
    damping_multiplier: float = 1.0
    adjust_damping_to_material: bool = False

    @classmethod
    def from_node(cls, n, first_order=False):
        c = cls(name=str(_get(n, "name", "")), collisions=bool(_get(n, "collisions", False)),
                graphics_only=bool(_get(n, "graphics-only", False)),
                position=_vec3(n, "position", [0, 0, 0]), velocity=_vec3(n, "velocity", [0, 0, 0]),
                rotation=_vec3(n, "rotation", [0, 0, 0]), filename=str(_get(n, "filename", "")),
                materials=list(_get(n, "materials", [])),
                element_classes_filename=_get(n, "element-classes-filename", None),
                self_collisions=bool(_get(n, "self-collisions", False)),
                num_solver_iters=int(_get(n, "num-solver-iters", 1)),
                num_local_collision_iters=int(_get(n, "num-local-collision-iters", 0)),
                solver_type=_options(n, "solver-type", SOLVER_TYPES, "Gauss-Seidel"),
                constraint_type=_options(n, "constraint-type", CONSTRAINT_TYPES, "Stable-Neohookean-Combined"),
                residual_policy=_options(n, "residual-policy", RESIDUAL_POLICIES, "Never"))
        if first_order:
            c.first_order = True
            c.damping_multiplier = float(_get(n, "damping-multiplier", 1.0))
            c.adjust_damping_to_material = bool(_get(n, "adjust-damping-to-material", False))
        if _get(n, "max-size", None) is not None:
            c.max_size = float(n["max-size"])
        if _get(n, "size", None) is not None:
            c.size = _vec3(n, "size", None)
        return c


@dataclass
class RigidSphereConfig:
    name: str = ""
    collisions: bool = False
    graphics_only: bool = False
    position: np.ndarray = field(default_factory=lambda: np.zeros(3))
    velocity: np.ndarray = field(default_factory=lambda: np.zeros(3))
    radius: float = 1.0
    density: float = 1000.0
    fixed: bool = False
    rotation: np.ndarray = field(default_factory=lambda: np.zeros(3))

    @classmethod
    def from_node(cls, n):
        return cls(name=str(_get(n, "name", "")), collisions=bool(_get(n, "collisions", False)),
                   graphics_only=bool(_get(n, "graphics-only", False)),
                   position=_vec3(n, "position", [0, 0, 0]), velocity=_vec3(n, "velocity", [0, 0, 0]),
                   radius=float(_get(n, "radius", 1.0)), density=float(_get(n, "density", 1000.0)),
                   fixed=bool(_get(n, "fixed", False)), rotation=_vec3(n, "rotation", [0, 0, 0]))


@dataclass
class RigidBoxConfig(RigidSphereConfig):
    size: np.ndarray = field(default_factory=lambda: np.ones(3))

    @classmethod
    def from_node(cls, n):
        b = RigidSphereConfig.from_node(n)
        return cls(**{**b.__dict__, "size": _vec3(n, "size", [1, 1, 1])})


@dataclass
class RigidCylinderConfig(RigidSphereConfig):
    height: float = 1.0

    @classmethod
    def from_node(cls, n):
        b = RigidSphereConfig.from_node(n)
        return cls(**{**b.__dict__, "height": float(_get(n, "height", 1.0))})


def eul_xyz_to_quat(deg):
    """Quaternion (x, y, z, w) of the rotation about x, then y, then z by the
    given angles in degrees (the reference's eulXYZ2Quat convention,
    src/utils/GeometryUtils.cpp:104-112)."""
    hx, hy, hz = (0.5 * np.radians(a) for a in deg)
    cx, sx, cy, sy, cz, sz = np.cos(hx), np.sin(hx), np.cos(hy), np.sin(hy), np.cos(hz), np.sin(hz)
    return np.array([sx * cy * cz - cx * sy * sz, cx * sy * cz + sx * cy * sz, cx * cy * sz - sx * sy * cz,
                     cx * cy * cz + sx * sy * sz])


SIM_MODES = {"Visualization": "Visualization", "AFAP": "AFAP", "Frame-by-frame": "Frame-by-frame"}
VISUALIZATIONS = {"None": "None", "Easy3D": "Easy3D", "VTK": "VTK"}


@dataclass
class SimulationConfig:
    name: str = ""
    description: str = ""
    time_step: float = 1e-3
    end_time: float = 10.0
    sim_mode: str = "Visualization"
    visualization: str = "VTK"
    g_accel: float = 9.81
    fps: float = 30.0
    collision_rate: float = 100.0
    materials: list = field(default_factory=list)
    objects: list = field(default_factory=list)

    @classmethod
    def from_node(cls, n):
        c = cls(name=str(_get(n, "name", "")), description=str(_get(n, "description", "")),
                time_step=float(_get(n, "time-step", 1e-3)), end_time=float(_get(n, "end-time", 10.0)),
                sim_mode=_options(n, "sim-mode", SIM_MODES, "Visualization"),
                visualization=_options(n, "visualization", VISUALIZATIONS, "VTK"),
                g_accel=float(_get(n, "g-accel", 9.81)), fps=float(_get(n, "fps", 30.0)),
                collision_rate=float(_get(n, "collision-rate", 100.0)))
        for on in _get(n, "objects", []):
            t = _get(on, "type", None)
            if t is None:
                raise ValueError("Type of object is needed!")
            if t == "XPBDMeshObject":
                c.objects.append(XPBDMeshObjectConfig.from_node(on))
            elif t == "FirstOrderXPBDMeshObject":
                c.objects.append(XPBDMeshObjectConfig.from_node(on, first_order=True))
            elif t == "RigidSphere":
                c.objects.append(RigidSphereConfig.from_node(on))
            elif t == "RigidBox":
                c.objects.append(RigidBoxConfig.from_node(on))
            elif t == "RigidCylinder":
                c.objects.append(RigidCylinderConfig.from_node(on))
            elif t in ("RigidMeshObject", "VirtuosoArm", "VirtuosoRobot"):
                raise NotImplementedError(f"object type {t!r} is not provided by the GB300 solver")
            else:
                raise ValueError(f"Unknown type of object! {t!r} is not a type of simulation object.")
        c.materials = [ElasticMaterialConfig.from_node(m) for m in _get(n, "materials", [])]
        return c


def load_config(path_or_text: str) -> tuple[SimulationConfig, str]:
    """(config, directory relative filenames resolve against)."""
    if "\n" in path_or_text:
        return SimulationConfig.from_node(yaml_lite.loads(path_or_text)), os.getcwd()
    return SimulationConfig.from_node(yaml_lite.load(path_or_text)), os.path.dirname(os.path.abspath(path_or_text))


def read_element_classes(path: str) -> np.ndarray:
    """FileUtils::readVectorFromFile<int> (include/utils/FileUtils.hpp:12-30):
    one integer per line, stopping at the first line that does not start with one."""
    out = []
    with open(path) as f:
        for line in f:
            tok = line.split()
            try:
                out.append(int(tok[0]))
            except (IndexError, ValueError):
                break
    return np.asarray(out, np.int64)


class XPBDObject:
    """One XPBDMeshObject: its placed mesh and its GPU solver."""

    def __init__(self, cfg: XPBDMeshObjectConfig, sim: "Simulation"):
        if cfg.self_collisions:
            raise NotImplementedError("self-collisions are not provided by the GB300 solver")
        self.cfg = cfg
        path = cfg.filename if os.path.isabs(cfg.filename) else os.path.join(sim.base_dir, cfg.filename)
        X, tets, faces = msh.read_msh(path)
        self.X = msh.place(X, faces, cfg.position, cfg.rotation, cfg.max_size, cfg.size)
        self.tets, self.faces = tets, faces
        T = tets.shape[0]
        mats = [sim.material(m) for m in cfg.materials] or [ElasticMaterialConfig()]
        cls = np.zeros(T, np.int64)
        if cfg.element_classes_filename:
            p = cfg.element_classes_filename
            p = p if os.path.isabs(p) else os.path.join(sim.base_dir, p)
            cls = read_element_classes(p)
            if cls.shape[0] != T:
                raise ValueError("Element classes file has a different number of elements than the mesh!")
        # classes past the material list take the last material (XPBDMeshObject.cpp:289-297)
        cls = np.minimum(cls, len(mats) - 1)
        self.E = np.array([mats[k].E for k in cls])
        self.nu = np.array([mats[k].nu for k in cls])
        self.rho = np.array([mats[k].density for k in cls])
        sc = sim.config
        self.solver = G.XPBDSolver(self.X, tets, faces if cfg.collisions else None, self.E, self.nu, self.rho,
                                   dt=sc.time_step, g_accel=sc.g_accel, collision_rate=sc.collision_rate,
                                   num_iters=cfg.num_solver_iters, solver_type=cfg.solver_type,
                                   constraint_type=cfg.constraint_type, residual_policy=cfg.residual_policy,
                                   num_local_collision_iters=cfg.num_local_collision_iters,
                                   first_order=int(cfg.first_order), damping_multiplier=cfg.damping_multiplier,
                                   adjust_damping_to_material=int(cfg.adjust_damping_to_material))
        if np.any(cfg.velocity != 0):
            self.solver.set_velocities(np.broadcast_to(cfg.velocity, self.X.shape))

    def positions(self):
        return self.solver.positions()

    def close(self):
        self.solver.close()


@dataclass
class Rigid:
    """A fixed rigid primitive: kind (G.SDF_*), pose, dimensions."""
    name: str
    kind: int
    position: np.ndarray
    quat: np.ndarray
    dims: np.ndarray
    collisions: bool


class Simulation:
    def __init__(self, config, base_dir: str | None = None):
        if isinstance(config, SimulationConfig):
            self.config, self.base_dir = config, base_dir or os.getcwd()
        else:
            self.config, d = load_config(config)
            self.base_dir = base_dir or d
        self.time = 0.0
        self.objects: dict[str, XPBDObject] = {}
        self.rigids: dict[str, Rigid] = {}
        self._setup = False

    def material(self, name: str) -> ElasticMaterialConfig:
        for m in self.config.materials:
            if m.name == name:
                return m
        raise ValueError(f"material {name!r} is not defined")

    def setup(self):
        assert not self._setup, "setup() called twice"
        self._setup = True
        for oc in self.config.objects:
            if oc.graphics_only:
                continue
            if isinstance(oc, RigidSphereConfig):
                if not oc.fixed:
                    raise NotImplementedError(f"rigid object {oc.name!r}: non-fixed rigid bodies (two-way "
                                              "coupling) are not provided; set `fixed: true`")
                if isinstance(oc, RigidBoxConfig):
                    kind, dims = G.SDF_BOX, np.asarray(oc.size, np.float64)
                elif isinstance(oc, RigidCylinderConfig):
                    kind, dims = G.SDF_CYLINDER, np.array([oc.radius, oc.height, 0.0])
                else:
                    kind, dims = G.SDF_SPHERE, np.array([oc.radius, 0.0, 0.0])
                rot = getattr(oc, "rotation", np.zeros(3))
                self.rigids[oc.name] = Rigid(oc.name, kind, oc.position.copy(), eul_xyz_to_quat(rot), dims,
                                             oc.collisions)
            else:
                self.objects[oc.name] = XPBDObject(oc, self)
        self._push_rigids()

    def _push_rigids(self):
        live = [r for r in self.rigids.values() if r.collisions]
        for o in self.objects.values():
            if o.cfg.collisions and live:
                o.solver.set_sdfs([r.kind for r in live], [r.position for r in live], [r.quat for r in live],
                                  [r.dims for r in live])

    def move_rigid(self, name: str, position, rotation_deg=None):
        """Kinematic motion of a fixed rigid object between steps."""
        r = self.rigids[name]
        r.position = np.asarray(position, np.float64)
        if rotation_deg is not None:
            r.quat = eul_xyz_to_quat(rotation_deg)
        self._push_rigids()

    def time_step(self):
        for o in self.objects.values():
            o.solver.step(1)
        self.time += self.config.time_step

    def update(self, max_steps: int | None = None):
        """Run until end-time (or max_steps steps); returns the steps taken."""
        start = time.perf_counter()
        n = 0
        while self.time < self.config.end_time and (max_steps is None or n < max_steps):
            if self.config.sim_mode == "Visualization":
                ahead = self.time - (time.perf_counter() - start)
                if ahead > 0:
                    time.sleep(ahead)
            self.time_step()
            n += 1
        for o in self.objects.values():
            o.solver.synchronize()
        return n

    def close(self):
        for o in self.objects.values():
            o.close()
        self.objects.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
