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

Rigid spheres, boxes and cylinders with `collisions: true` collide with
every XPBD object that has `collisions: true`, as SDFs in the solver
(orientation from `rotation`, RigidObject.cpp:12-14, whose degrees-to-radians
factor is 3.1415/180). Fixed ones are static and can be moved between steps
(move_rigid). Free ones (`fixed: false`) are the solver's rigid bodies: mass
and inertia from `density` and the dimensions (RigidPrimitives.cpp), the
initial `velocity` and `angular-velocity`, two-way coupling with the XPBD
object in the solve, gravity and the angular Euler step after it
(RigidObject.cpp:41-77). A free body without collisions only falls; it is
integrated here on the host. The reference only builds graphics for
`visualization`; there is no graphics here and the key is read and ignored.

`self-collisions: true` turns on the solver's self-collision detection and
constraints (XPBDMeshObject.cpp:719-762).

Not provided (each raises NotImplementedError naming the key): a free rigid
body colliding with more than one XPBD object, rigid meshes and the Virtuoso
robot objects.
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
    angular_velocity: np.ndarray = field(default_factory=lambda: np.zeros(3))

    @classmethod
    def from_node(cls, n):
        return cls(name=str(_get(n, "name", "")), collisions=bool(_get(n, "collisions", False)),
                   graphics_only=bool(_get(n, "graphics-only", False)),
                   position=_vec3(n, "position", [0, 0, 0]), velocity=_vec3(n, "velocity", [0, 0, 0]),
                   radius=float(_get(n, "radius", 1.0)), density=float(_get(n, "density", 1000.0)),
                   fixed=bool(_get(n, "fixed", False)), rotation=_vec3(n, "rotation", [0, 0, 0]),
                   angular_velocity=_vec3(n, "angular-velocity", [0, 0, 0]))

    def mass_inertia(self):
        """RigidSphere's mass and diagonal inertia (RigidPrimitives.cpp:9-20, pi as 3.1415)."""
        m = 4.0 / 3.0 * 3.1415 * self.radius * self.radius * self.radius * self.density
        i = 2.0 / 5.0 * m * self.radius * self.radius
        return m, np.array([i, i, i])


@dataclass
class RigidBoxConfig(RigidSphereConfig):
    size: np.ndarray = field(default_factory=lambda: np.ones(3))

    @classmethod
    def from_node(cls, n):
        b = RigidSphereConfig.from_node(n)
        return cls(**{**b.__dict__, "size": _vec3(n, "size", [1, 1, 1])})

    def mass_inertia(self):
        """RigidBox (RigidPrimitives.cpp:39-48)."""
        sx, sy, sz = self.size
        m = sx * sy * sz * self.density
        return m, np.array([1.0 / 12.0 * m * (sy * sy + sz * sz), 1.0 / 12.0 * m * (sx * sx + sz * sz),
                            1.0 / 12.0 * m * (sx * sx + sy * sy)])


@dataclass
class RigidCylinderConfig(RigidSphereConfig):
    height: float = 1.0

    @classmethod
    def from_node(cls, n):
        b = RigidSphereConfig.from_node(n)
        return cls(**{**b.__dict__, "height": float(_get(n, "height", 1.0))})

    def mass_inertia(self):
        """RigidCylinder (RigidPrimitives.cpp:86-94)."""
        r, h = self.radius, self.height
        m = 3.1415 * r * r * h * self.density
        return m, np.array([1.0 / 12.0 * m * (3 * r * r + h * h), 1.0 / 12.0 * m * (3 * r * r + h * h),
                            1.0 / 2.0 * m * r * r])


def eul_xyz_to_quat(deg, rad_per_deg=np.pi / 180.0):
    """Quaternion (x, y, z, w) of the rotation about x, then y, then z by the
    given angles in degrees (the reference's eulXYZ2Quat convention,
    src/utils/GeometryUtils.cpp:104-112)."""
    hx, hy, hz = (0.5 * a * rad_per_deg for a in deg)
    cx, sx, cy, sy, cz, sz = np.cos(hx), np.sin(hx), np.cos(hy), np.sin(hy), np.cos(hz), np.sin(hz)
    return np.array([sx * cy * cz - cx * sy * sz, cx * sy * cz + sx * cy * sz, cx * cy * sz - sx * sy * cz,
                     cx * cy * cz + sx * sy * sz])


def rigid_quat(deg):
    """A rigid object's initial orientation: its `rotation` in degrees turned
    to radians with the reference's factor 3.1415/180 (RigidObject.cpp:12-14)."""
    return eul_xyz_to_quat(deg, 3.1415 / 180.0)


class FreeBody:
    """RigidObject::update / velocityUpdate (RigidObject.cpp:41-77) for a free
    body that collides with nothing, on the host; the solver runs the same
    steps on the device for free bodies that collide."""

    def __init__(self, p, q, v, w, m, inertia):
        self.p, self.q = np.array(p, float), np.array(q, float)
        self.v, self.w = np.array(v, float), np.array(w, float)
        self.p_prev, self.q_prev = self.p.copy(), self.q.copy()
        self.m, self.I = float(m), np.asarray(inertia, float)

    @staticmethod
    def _mult(a, b):
        return np.array([a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1],
                         a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2],
                         a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0],
                         a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2]])

    @staticmethod
    def _rot(v, q):
        u = q[:3]
        return 2 * u.dot(v) * u + (2 * q[3] * q[3] - 1) * v + 2 * q[3] * np.cross(u, v)

    @staticmethod
    def _inv(q):
        return np.array([-q[0], -q[1], -q[2], q[3]]) / q.dot(q)

    def update(self, dt, g):
        self.v = self.v + dt * np.array([0.0, 0.0, -self.m * g]) / self.m
        self.p = self.p + dt * self.v
        wb = self._rot(self.w, self._inv(self.q))
        wb = wb + dt * (1.0 / self.I) * (0.0 - np.cross(wb, self.I * wb))
        self.w = self._rot(wb, self.q)
        self.q = self.q + 0.5 * dt * self._mult(np.append(self.w, 0.0), self.q)
        self.q = self.q / np.linalg.norm(self.q)

    def velocity_update(self, dt):
        self.v = (self.p - self.p_prev) / dt
        dq = self._mult(self.q, self._inv(self.q_prev))
        self.w = 2 / dt * dq[:3] * (-1.0 if dq[3] < 0 else 1.0)
        self.p_prev, self.q_prev = self.p.copy(), self.q.copy()


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
                                   adjust_damping_to_material=int(cfg.adjust_damping_to_material),
                                   self_collisions=int(cfg.self_collisions))
        if np.any(cfg.velocity != 0):
            self.solver.set_velocities(np.broadcast_to(cfg.velocity, self.X.shape))

    def positions(self):
        return self.solver.positions()

    def close(self):
        self.solver.close()


@dataclass
class Rigid:
    """A rigid primitive: kind (G.SDF_*), pose, dimensions; free bodies also
    carry mass, inertia and their initial velocities (the solver, or a
    FreeBody when it collides with nothing, holds the live state)."""
    name: str
    kind: int
    position: np.ndarray
    quat: np.ndarray
    dims: np.ndarray
    collisions: bool
    fixed: bool = True
    mass: float = 0.0
    inertia: np.ndarray = field(default_factory=lambda: np.zeros(3))
    velocity: np.ndarray = field(default_factory=lambda: np.zeros(3))
    angular_velocity: np.ndarray = field(default_factory=lambda: np.zeros(3))
    host_body: FreeBody | None = None


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
                if isinstance(oc, RigidBoxConfig):
                    kind, dims = G.SDF_BOX, np.asarray(oc.size, np.float64)
                elif isinstance(oc, RigidCylinderConfig):
                    kind, dims = G.SDF_CYLINDER, np.array([oc.radius, oc.height, 0.0])
                else:
                    kind, dims = G.SDF_SPHERE, np.array([oc.radius, 0.0, 0.0])
                rot = getattr(oc, "rotation", np.zeros(3))
                r = Rigid(oc.name, kind, oc.position.copy(), rigid_quat(rot), dims, oc.collisions, oc.fixed)
                if not oc.fixed:
                    r.mass, r.inertia = oc.mass_inertia()
                    r.velocity, r.angular_velocity = oc.velocity.copy(), oc.angular_velocity.copy()
                    if not oc.collisions:
                        r.host_body = FreeBody(r.position, r.quat, r.velocity, r.angular_velocity, r.mass, r.inertia)
                self.rigids[oc.name] = r
            else:
                self.objects[oc.name] = XPBDObject(oc, self)
        colliding = [o for o in self.objects.values() if o.cfg.collisions]
        if len(colliding) > 1 and any(not r.fixed and r.collisions for r in self.rigids.values()):
            raise NotImplementedError("a free rigid body colliding with more than one XPBD object is not provided")
        self._pushed = False
        self._push_rigids()

    def _push_rigids(self):
        live = [r for r in self.rigids.values() if r.collisions]
        for o in self.objects.values():
            if o.cfg.collisions and live:
                if self._pushed:
                    # setting the SDFs drops the free bodies: carry their live state over
                    for slot, r in enumerate(live):
                        if not r.fixed:
                            r.position, r.quat, r.velocity, r.angular_velocity = o.solver.rigid_body(slot)
                o.solver.set_sdfs([r.kind for r in live], [r.position for r in live], [r.quat for r in live],
                                  [r.dims for r in live])
                for slot, r in enumerate(live):
                    if not r.fixed:
                        o.solver.set_rigid_body(slot, r.mass, r.inertia, r.velocity, r.angular_velocity)
        self._pushed = True

    def move_rigid(self, name: str, position, rotation_deg=None):
        """Kinematic motion of a fixed rigid object between steps."""
        r = self.rigids[name]
        if not r.fixed:
            raise ValueError(f"rigid object {name!r} is free: the solver moves it")
        r.position = np.asarray(position, np.float64)
        if rotation_deg is not None:
            r.quat = rigid_quat(rotation_deg)
        self._push_rigids()

    def rigid_state(self, name: str):
        """(position, orientation (x, y, z, w), velocity, angular velocity) of a rigid object."""
        r = self.rigids[name]
        if r.host_body is not None:
            b = r.host_body
            return b.p.copy(), b.q.copy(), b.v.copy(), b.w.copy()
        if not r.fixed:
            live = [x for x in self.rigids.values() if x.collisions]
            for o in self.objects.values():
                if o.cfg.collisions:
                    return o.solver.rigid_body(live.index(r))
        return r.position.copy(), r.quat.copy(), np.zeros(3), np.zeros(3)

    def time_step(self):
        for o in self.objects.values():
            o.solver.step(1)
        # free bodies that collide with nothing: RigidObject::update, velocityUpdate
        for r in self.rigids.values():
            if r.host_body is not None:
                r.host_body.update(self.config.time_step, self.config.g_accel)
                r.host_body.velocity_update(self.config.time_step)
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
