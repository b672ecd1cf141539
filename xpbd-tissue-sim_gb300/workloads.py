"""Synthetic workloads: the meshes, materials and boundary conditions of the
benchmark configurations, built with the library's own grid generator.

  cube   unit cube, 10x10x10 hexes x 5 tets (5,000 tets, 1,331 vertices),
         E=3e3 Pa, nu=0.45, rho=1000, bottom (z=min) fixed, initial positions
         rest + U(-1e-3, 1e-3) m (numpy PCG64, seeded)
  beam   0.5 x 0.05 x 0.05 m beam, 100x10x10 hexes (50,000 tets, 12,221
         vertices) along y, E=1e4, nu=0.49, y=min end clamped; a rigid sphere of
         radius 0.03 m starts over the beam midpoint 2 mm into the top face and
         descends at 0.05 m/s. The reference's un-averaged Jacobi diverges on
         this nearly incompressible beam (the FP64 oracle moves vertices by
         0.42 m after 20 steps and 19 km after 50), so the workload defaults to
         coloured Gauss-Seidel; jacobi=True selects the reference's Jacobi.
  block  64^3 hexes (1,310,720 tets, 274,625 vertices) on a 0.1 m cube, per-tet
         E log-uniform in [1e3, 1e5] (seeded), nu=0.45, bottom fixed, top face
         kinematically raised by 1 cm linearly over 100 steps

Boundary conditions follow the reference's patterns: clamp by min-y
(src/simulation/BeamSimulation.cpp:31-34), fix the bottom by min-z
(src/simulation/GraspingSimulation.cpp:41), kinematic vertices as fixVertex plus
a prescribed position (GraspingSimulation.cpp:155,241).

The builders take the grid generator as `mesher` (the library's
xpbd_gb300.grid_mesh by default); the CPU reference arm passes the oracle's
own generator, so building a workload there loads nothing of the GPU library.
This module imports xpbd_gb300 only inside the functions that make solvers.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# solver-type codes of the C ABI (XPBD_SOLVER_GAUSS_SEIDEL, XPBD_SOLVER_JACOBI)
GAUSS_SEIDEL = 0
JACOBI = 1


def _mesher(mesher):
    if mesher is not None:
        return mesher
    import xpbd_gb300 as G
    return G.grid_mesh


@dataclass
class Workload:
    name: str
    X: np.ndarray
    tets: np.ndarray
    faces: np.ndarray
    E: np.ndarray
    nu: np.ndarray
    rho: np.ndarray
    fixed: np.ndarray
    x0: np.ndarray                       # initial positions
    dt: float = 1e-3
    g: float = 9.81
    iters: int = 10
    solver: int = GAUSS_SEIDEL
    steps: int = 100
    sphere_r: float = 0.0
    sphere_c0: np.ndarray | None = None  # centre at t = 0
    sphere_v: np.ndarray | None = None   # centre velocity
    kin_idx: np.ndarray | None = None    # kinematic vertex group
    kin_dir: np.ndarray | None = None    # full prescribed displacement
    kin_ramp_steps: int = 100
    collision_rate: float = 100.0
    meta: dict = field(default_factory=dict)

    @property
    def V(self):
        return self.X.shape[0]

    @property
    def T(self):
        return self.tets.shape[0]

    def sphere_centre(self, t: float) -> np.ndarray:
        return self.sphere_c0 + self.sphere_v * t

    def kin_offset(self, step: int) -> np.ndarray:
        return self.kin_dir * min(step / self.kin_ramp_steps, 1.0)


def cube(n: int = 10, seed: int = 0, noise: float = 1e-3, mesher=None) -> Workload:
    X, tets, faces = _mesher(mesher)(n, n, n, 1.0 / n)
    rng = np.random.default_rng(seed)
    x0 = X + rng.uniform(-noise, noise, X.shape)
    T = tets.shape[0]
    return Workload("cube", X, tets, faces, np.full(T, 3e3), np.full(T, 0.45), np.full(T, 1000.0),
                    fixed=X[:, 2] == X[:, 2].min(), x0=x0, iters=10, solver=GAUSS_SEIDEL, steps=200)


def beam(nl: int = 100, nw: int = 10, nh: int = 10, length: float = 0.5, with_sphere: bool = True,
         jacobi: bool = False, mesher=None) -> Workload:
    h = length / nl
    X, tets, faces = _mesher(mesher)(nw, nl, nh, h)
    T = tets.shape[0]
    top = X[:, 2].max()
    r = 0.03
    c0 = np.array([X[:, 0].max() / 2, X[:, 1].max() / 2, top + r - 0.002])
    w = Workload("beam", X, tets, faces, np.full(T, 1e4), np.full(T, 0.49), np.full(T, 1000.0),
                 fixed=X[:, 1] == X[:, 1].min(), x0=X.copy(), iters=20,
                 solver=JACOBI if jacobi else GAUSS_SEIDEL, steps=500)
    if with_sphere:
        w.sphere_r = r
        w.sphere_c0 = c0
        w.sphere_v = np.array([0.0, 0.0, -0.05])
    return w


def block(n: int = 64, size: float = 0.1, seed: int = 0, E_range=(1e3, 1e5), iters: int = 30,
          mesher=None) -> Workload:
    X, tets, faces = _mesher(mesher)(n, n, n, size / n)
    T = tets.shape[0]
    rng = np.random.default_rng(seed)
    E = np.exp(rng.uniform(np.log(E_range[0]), np.log(E_range[1]), T))
    zmin, zmax = X[:, 2].min(), X[:, 2].max()
    top = np.nonzero(X[:, 2] == zmax)[0].astype(np.int32)
    return Workload("block", X, tets, faces, E, np.full(T, 0.45), np.full(T, 1000.0),
                    fixed=X[:, 2] == zmin, x0=X.copy(), iters=iters, solver=GAUSS_SEIDEL, steps=100,
                    kin_idx=top, kin_dir=np.array([0.0, 0.0, 0.01]), kin_ramp_steps=100)


@dataclass
class Batch:
    """Independent instances advanced together (concatenated in instance order)."""
    instances: list
    name: str = "batched"

    @property
    def T(self):
        return sum(w.T for w in self.instances)

    @property
    def V(self):
        return sum(w.V for w in self.instances)

    @property
    def iters(self):
        return self.instances[0].iters

    @property
    def dt(self):
        return self.instances[0].dt


def batched(n: int = 256, seed: int = 0, t_range=(2_000, 100_000), iters: int = 20,
            solver: int = GAUSS_SEIDEL, mesher=None) -> Batch:
    """n cube/beam instances with tet counts log-uniform in t_range (seeded grid
    dims, T = 5 nx ny nz), E log-uniform in [1e3, 1e5] Pa, nu in [0.40, 0.49],
    rho 1000, bottom fixed, 1-4 seeded spheres descending at 0.05 m/s onto the
    top surface."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        target = np.exp(rng.uniform(np.log(t_range[0]), np.log(t_range[1]))) / 5.0
        if rng.random() < 0.5:  # cube
            m = max(2, int(round(target ** (1 / 3))))
            nx, ny, nz = m, m, m
        else:  # beam: length 4x the section
            m = max(2, int(round((target / 4) ** (1 / 3))))
            nx, ny, nz = m, 4 * m, m
        h = 0.05 / nx
        X, tets, faces = _mesher(mesher)(nx, ny, nz, h)
        T = tets.shape[0]
        E = np.full(T, float(np.exp(rng.uniform(np.log(1e3), np.log(1e5)))))
        nu = np.full(T, float(rng.uniform(0.40, 0.49)))
        w = Workload(f"inst{k}", X, tets, faces, E, nu, np.full(T, 1000.0), fixed=X[:, 2] == X[:, 2].min(),
                     x0=X.copy(), iters=iters, solver=solver, steps=100)
        ns = int(rng.integers(1, 5))
        top = X[:, 2].max()
        r = rng.uniform(0.2, 0.4, ns) * X[:, 0].max()
        cx = rng.uniform(0.2, 0.8, ns) * X[:, 0].max()
        cy = rng.uniform(0.2, 0.8, ns) * X[:, 1].max()
        w.meta["spheres"] = (np.stack([cx, cy, top + r - 0.1 * r], 1), r)
        w.sphere_r = float(r[0])
        w.sphere_c0 = w.meta["spheres"][0][0]
        w.sphere_v = np.array([0.0, 0.0, -0.05])
        out.append(w)
    return Batch(out)


def make_batch_solver(b: Batch, **params):
    """One context holding every instance of the batch."""
    import xpbd_gb300 as G
    w0 = b.instances[0]
    kw = dict(dt=w0.dt, g_accel=w0.g, num_iters=w0.iters, solver_type=w0.solver, collision_rate=w0.collision_rate)
    kw.update(params)
    s = G.XPBDSolver(instances=[(w.X, w.tets, w.faces, w.E, w.nu, w.rho) for w in b.instances], **kw)
    s.fix_vertices(np.concatenate([w.fixed for w in b.instances]))
    s.set_positions(np.concatenate([w.x0 for w in b.instances]))
    return s


def drive_batch(s, b: Batch):
    """Sphere centres of every instance at the solver's current time."""
    t = s.time
    for k, w in enumerate(b.instances):
        c, r = w.meta["spheres"]
        s.set_spheres(c + w.sphere_v * t, r, instance=k)


def make_solver(w: Workload, **params):
    """GPU solver set up for a workload: fixed vertices, kinematic group,
    initial positions, spheres."""
    import xpbd_gb300 as G
    kw = dict(dt=w.dt, g_accel=w.g, num_iters=w.iters, solver_type=w.solver, collision_rate=w.collision_rate)
    kw.update(params)
    faces = w.faces if w.sphere_r > 0 else None
    s = G.XPBDSolver(w.X, w.tets, faces, w.E, w.nu, w.rho, **kw)
    s.fix_vertices(w.fixed)
    s.set_positions(w.x0)
    if w.kin_idx is not None:
        s.set_kinematic_group(w.kin_idx)
    return s


def drive_gpu(s, w: Workload, step: int):
    """Per-step kinematic inputs (sphere centre, kinematic offset) for step `step`
    at the solver's current time."""
    if w.sphere_r > 0:
        s.set_spheres(w.sphere_centre(s.time), [w.sphere_r])
    if w.kin_idx is not None:
        s.set_kinematic_offset(w.kin_offset(step))
