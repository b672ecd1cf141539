"""ctypes wrapper of the XPBD oracle (oracle/xpbd_oracle.hpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; the shipped library never uses it.
Physics parity is unpinned (the reference ships no golden vectors and cannot be
built without Eigen/yaml-cpp/gmsh); the grid generator is pinned against the
reference's own cube*.msh outputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libxpbd_oracle.so")

GAUSS_SEIDEL, JACOBI, COLOURED_GS = 0, 1, 2
COMBINED, SEPARATE = 0, 1

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, I, LL, D = C.c_void_p, C.c_int, C.c_longlong, C.c_double
        L.xo_create.restype = P
        L.xo_create.argtypes = [I, LL, P, LL, P, LL, P, P, P, P, D, D, I, I, I]
        for name in ["xo_destroy", "xo_velocity_update", "xo_iterate"]:
            getattr(L, name).argtypes = [P]
        L.xo_time_steps.restype = D
        L.xo_time_steps.argtypes = [P, I, I]
        L.xo_time.restype = D
        L.xo_time.argtypes = [P]
        L.xo_residual_norm.restype = D
        L.xo_residual_norm.argtypes = [P]
        L.xo_strain_energy.restype = D
        L.xo_strain_energy.argtypes = [P]
        L.xo_set_collision_rate.argtypes = [P, D]
        L.xo_grid_counts.argtypes = [I, I, I, P, P, P]
        L.xo_grid_mesh.argtypes = [I, I, I, D, D, D, P, P, P, I]
        L.xo_greedy_colour.argtypes = [LL, I, P, LL, P]
        L.xo_greedy_colour.restype = I
        L.xo_set_rel_tol.argtypes = [P, D]
        L.xo_update_start.argtypes = [P, P, P, I]
        L.xo_last_r_plain.argtypes = [P]
        L.xo_last_r_plain.restype = D
        L.xo_iters_done.argtypes = [P]
        L.xo_iters_done.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def grid_mesh(w: int, l: int, h: int, ex: float, ey: float | None = None, ez: float | None = None,
              split: int = 0):
    """Hex grid split into 5 tets per hex (restates MeshUtils::createBeamMsh,
    src/utils/MeshUtils.cpp:424-660). split=0: alternating split of the current
    source; split=1: the uniform split that wrote resource/cube/cube{2,4}.msh.
    Returns X (V,3) float64, tets (T,4) int32, faces (F,3) int32."""
    ey = ex if ey is None else ey
    ez = ex if ez is None else ez
    L = lib()
    V, T, F = C.c_longlong(), C.c_longlong(), C.c_longlong()
    L.xo_grid_counts(w, l, h, C.byref(V), C.byref(T), C.byref(F))
    X = np.zeros((V.value, 3), np.float64)
    tets = np.zeros((T.value, 4), np.int32)
    faces = np.zeros((F.value, 3), np.int32)
    L.xo_grid_mesh(w, l, h, ex, ey, ez, _p(X), _p(tets), _p(faces), int(split))
    return X, tets, faces


def greedy_colour(items: np.ndarray, n_vertices: int):
    items = np.ascontiguousarray(items, np.int32)
    out = np.zeros(items.shape[0], np.int32)
    n = lib().xo_greedy_colour(items.shape[0], items.shape[1], _p(items), n_vertices, _p(out))
    return n, out


class Oracle:
    """One XPBD mesh object with its solver (XPBDMeshObject_ + XPBDSolver)."""

    def __init__(self, X, tets, faces, E, nu, rho, dt=1e-3, g=9.81, num_iter=1,
                 solver=GAUSS_SEIDEL, ckind=COMBINED, precision=64):
        L = lib()
        self.X = np.ascontiguousarray(X, np.float64)
        self.tets = np.ascontiguousarray(tets, np.int32)
        self.faces = np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
        self.V, self.T, self.F = self.X.shape[0], self.tets.shape[0], self.faces.shape[0]
        bc = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), (self.T,)))
        self._E, self._nu, self._rho = bc(E), bc(nu), bc(rho)
        self.h = L.xo_create(precision, self.V, _p(self.X), self.T, _p(self.tets), self.F, _p(self.faces),
                             _p(self._E), _p(self._nu), _p(self._rho), dt, g, num_iter, solver, ckind)
        self.L = L

    def close(self):
        if self.h:
            self.L.xo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # state
    def _get(self, fn, shape):
        out = np.zeros(shape, np.float64)
        getattr(self.L, fn)(C.c_void_p(self.h), _p(out))
        return out

    def positions(self):
        return self._get("xo_get_positions", (self.V, 3))

    def prev_positions(self):
        return self._get("xo_get_prev_positions", (self.V, 3))

    def velocities(self):
        return self._get("xo_get_velocities", (self.V, 3))

    def masses(self):
        return self._get("xo_get_masses", (self.V,))

    def lambdas(self):
        return self._get("xo_get_lambda", (self.T, 2))

    def set_lambdas(self, lam):
        lam = np.ascontiguousarray(lam, np.float64)
        self.L.xo_set_lambda(C.c_void_p(self.h), _p(lam))

    def set_positions(self, x):
        x = np.ascontiguousarray(x, np.float64)
        self.L.xo_set_positions(C.c_void_p(self.h), _p(x))

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, np.float64)
        self.L.xo_set_velocities(C.c_void_p(self.h), _p(v))

    def set_fixed(self, mask):
        m = np.ascontiguousarray(mask, np.uint8)
        self.L.xo_set_fixed(C.c_void_p(self.h), _p(m))

    def tet_data(self):
        Q = np.zeros((self.T, 9)); vol = np.zeros(self.T); ad = np.zeros(self.T)
        ah = np.zeros(self.T); gm = np.zeros(self.T)
        self.L.xo_get_tet_data(C.c_void_p(self.h), _p(Q), _p(vol), _p(ad), _p(ah), _p(gm))
        return Q, vol, ad, ah, gm

    def set_num_iter(self, n):
        self.L.xo_set_num_iter(C.c_void_p(self.h), int(n))

    # collisions
    def set_collision_rate(self, rate):
        self.L.xo_set_collision_rate(C.c_void_p(self.h), float(rate))

    def set_spheres(self, centers, radii):
        c = np.ascontiguousarray(centers, np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(radii, np.float64).reshape(-1)
        self.L.xo_set_spheres(C.c_void_p(self.h), len(r), _p(c), _p(r))

    def add_attachment(self, vertex, target):
        t = np.ascontiguousarray(target, np.float64)
        self.L.xo_add_attachment(C.c_void_p(self.h), int(vertex), _p(t))

    def set_attachment_target(self, attachment, target):
        t = np.ascontiguousarray(target, np.float64)
        self.L.xo_set_attachment_target(C.c_void_p(self.h), int(attachment), _p(t))

    def set_prims(self, kinds, positions, quats, dims):
        """Fixed SDF primitives: kinds 0 sphere, 1 box, 2 cylinder; quats (x, y, z, w)."""
        k = np.ascontiguousarray(kinds, np.int32).reshape(-1)
        n = k.size
        p = np.ascontiguousarray(positions, np.float64).reshape(n, 3)
        q = np.ascontiguousarray(quats, np.float64).reshape(n, 4)
        d = np.ascontiguousarray(dims, np.float64).reshape(n, 3)
        self.L.xo_set_prims(C.c_void_p(self.h), n, _p(k), _p(p), _p(q), _p(d))

    def set_rigid_body(self, prim, position, quat, mass, inertia, velocity=(0, 0, 0), angular_velocity=(0, 0, 0)):
        """Primitive `prim` (after set_prims) becomes a free rigid body."""
        a = [np.ascontiguousarray(v, np.float64) for v in (position, quat, inertia, velocity, angular_velocity)]
        self.L.xo_set_rigid_body(C.c_void_p(self.h), int(prim), _p(a[0]), _p(a[1]), C.c_double(mass), _p(a[2]),
                                 _p(a[3]), _p(a[4]))

    def rigid_body(self, prim):
        """(position, quaternion (x, y, z, w), velocity, angular velocity)."""
        out = np.zeros(13)
        self.L.xo_get_rigid_body(C.c_void_p(self.h), int(prim), _p(out))
        return out[:3], out[3:7], out[7:10], out[10:13]

    def enable_self_collisions(self):
        self.L.xo_enable_self_collisions(C.c_void_p(self.h))

    def self_contacts(self):
        """rows of (surface vertex, surface face, lambda) found by the last detection."""
        n = self.L.xo_num_self_contacts(C.c_void_p(self.h))
        out = np.zeros((n, 3))
        if n:
            self.L.xo_get_self_contacts(C.c_void_p(self.h), _p(out))
        return out

    def self_contact_eval(self, v, f):
        """C and its 12-entry gradient for vertex v against face f at the current positions."""
        g = np.zeros(12)
        self.L.xo_self_contact_eval.restype = C.c_double
        c = self.L.xo_self_contact_eval(C.c_void_p(self.h), int(v), int(f), _p(g))
        return c, g

    def detect(self):
        return self.L.xo_detect(C.c_void_p(self.h))

    def contacts(self):
        n = self.L.xo_num_contacts(C.c_void_p(self.h))
        out = np.zeros((n, 12))
        if n:
            self.L.xo_get_contacts(C.c_void_p(self.h), _p(out))
        return out

    def set_contacts(self, rows):
        rows = np.ascontiguousarray(rows, np.float64).reshape(-1, 12)
        self.L.xo_set_contacts(C.c_void_p(self.h), rows.shape[0], _p(rows))

    def set_kinematic_group(self, idx):
        idx = np.ascontiguousarray(idx, np.int32)
        self.L.xo_set_kinematic_group(C.c_void_p(self.h), len(idx), _p(idx))

    def set_kinematic_offset(self, off):
        off = np.ascontiguousarray(off, np.float64)
        self.L.xo_set_kinematic_offset(C.c_void_p(self.h), _p(off))

    # stepping
    def update(self, record=False):
        self.L.xo_update(C.c_void_p(self.h), int(record))

    def update_warm(self, lam0, record=False, fallback=True):
        """Warm-started update from multipliers lam0 (T x 2, dev/hyd); returns
        True when the warm start was kept (not rejected by the residual test)."""
        lam0 = np.ascontiguousarray(lam0, np.float64)
        return bool(self.L.xo_update_warm(C.c_void_p(self.h), _p(lam0), int(record), int(fallback)))

    def update_start(self, dx0=None, lam0=None, record=False):
        """Update from a given start (warm-start experiments): positions moved
        by dx0 (V x 3) after the inertial move, multipliers starting at lam0
        (T x 2); last_r_plain() is ||r(x_pred, 0)||."""
        d = None if dx0 is None else np.ascontiguousarray(dx0, np.float64)
        l = None if lam0 is None else np.ascontiguousarray(lam0, np.float64)
        self.L.xo_update_start(C.c_void_p(self.h), _p(d), _p(l), int(record))

    def last_r_plain(self):
        return self.L.xo_last_r_plain(C.c_void_p(self.h))

    def set_rel_tol(self, tol):
        """Convergence measurement: update() stops its sweeps once ||r|| <=
        tol * ||r(x_pred, 0)|| (at most num_iter sweeps); 0 turns it off."""
        self.L.xo_set_rel_tol(C.c_void_p(self.h), float(tol))

    def iters_done(self):
        """Sweeps the last update() ran."""
        return self.L.xo_iters_done(C.c_void_p(self.h))

    def velocity_update(self):
        self.L.xo_velocity_update(self.h)

    def iterate(self):
        self.L.xo_iterate(self.h)

    def time_steps(self, n, record=False):
        return self.L.xo_time_steps(self.h, int(n), int(record))

    @property
    def time(self):
        return self.L.xo_time(self.h)

    def res_history(self):
        n = self.L.xo_res_history(C.c_void_p(self.h), None)
        out = np.zeros(n)
        if n:
            self.L.xo_res_history(C.c_void_p(self.h), _p(out))
        return out

    def residual_norm(self):
        return self.L.xo_residual_norm(self.h)

    def constraint_residual(self):
        return self._get("xo_constraint_residual", (2 * self.T,))

    def strain_energy(self):
        return self.L.xo_strain_energy(self.h)

    def set_order(self, order):
        """Replay a given Gauss-Seidel order (a permutation of the tets)."""
        order = np.ascontiguousarray(order, np.int32)
        if self.L.xo_set_order(C.c_void_p(self.h), len(order), _p(order)) != 0:
            raise ValueError("not a permutation of the tets")

    def set_first_order(self, damping_multiplier=1.0, adjust=False):
        """FirstOrderXPBDMeshObject: alpha~ = alpha/dt, vertex damping as inertia."""
        E = np.ascontiguousarray(np.broadcast_to(self._E, (self.T,)), np.float64)
        nu = np.ascontiguousarray(np.broadcast_to(self._nu, (self.T,)), np.float64)
        self.L.xo_set_first_order(C.c_void_p(self.h), C.c_double(damping_multiplier), int(adjust), _p(E), _p(nu))

    def set_local_iterations(self, iters, order=None):
        """num-local-collision-iters; `order` (a tet permutation) is the tet
        order of the coloured local passes."""
        if order is None:
            st = self.L.xo_set_local(C.c_void_p(self.h), int(iters), 0, None)
        else:
            order = np.ascontiguousarray(order, np.int32)
            st = self.L.xo_set_local(C.c_void_p(self.h), int(iters), len(order), _p(order))
        if st != 0:
            raise ValueError("bad local iteration settings")

    def local_tets(self):
        """Tets gathered for the local collision passes, duplicates included."""
        n = self.L.xo_local_tets(C.c_void_p(self.h), None)
        out = np.zeros(n, np.int32)
        if n:
            self.L.xo_local_tets(C.c_void_p(self.h), _p(out))
        return out

    def tet_order(self):
        n = self.L.xo_tet_order(C.c_void_p(self.h), None)
        out = np.zeros(n, np.int32)
        if n:
            self.L.xo_tet_order(C.c_void_p(self.h), _p(out))
        return out


PRIM_SPHERE, PRIM_BOX, PRIM_CYLINDER = 0, 1, 2


def prim_eval(kind, position, quat, dims, x, precision=64):
    """(sdf, gx, gy, gz) of one SDF primitive at point x."""
    out = np.zeros(4)
    pos = np.ascontiguousarray(position, np.float64)
    q = np.ascontiguousarray(quat, np.float64)
    d = np.ascontiguousarray(dims, np.float64)
    xx = np.ascontiguousarray(x, np.float64)
    lib().xo_prim_eval(int(precision), int(kind), _p(pos), _p(q), _p(d), _p(xx), _p(out))
    return out


def read_msh41(path_or_text: str):
    """Minimal gmsh 4.1 ASCII reader for the node/triangle/tet sections the
    reference's loader consumes (src/utils/MeshUtils.cpp:92-219): returns
    X (V,3), faces (F,3) 0-based, tets (T,4) 0-based."""
    text = path_or_text
    if "\n" not in path_or_text and os.path.exists(path_or_text):
        with open(path_or_text) as f:
            text = f.read()
    lines = [ln.strip() for ln in text.splitlines()]
    i = lines.index("$Nodes")
    nblocks, nnodes = map(int, lines[i + 1].split()[:2])
    i += 2
    tags, coords = [], []
    for _ in range(nblocks):
        _, _, _, n = map(int, lines[i].split())
        i += 1
        tags.extend(int(lines[i + k]) for k in range(n))
        coords.extend([float(v) for v in lines[i + n + k].split()[:3]] for k in range(n))
        i += 2 * n
    X = np.zeros((max(tags), 3))
    X[np.array(tags) - 1] = np.array(coords)
    i = lines.index("$Elements")
    nblocks = int(lines[i + 1].split()[0])
    i += 2
    faces, tets = [], []
    for _ in range(nblocks):
        _, _, etype, n = map(int, lines[i].split())
        i += 1
        rows = [list(map(int, lines[i + k].split()[1:])) for k in range(n)]
        i += n
        if etype == 2:
            faces.extend(rows)
        elif etype == 4:
            tets.extend(rows)
    return X, np.array(faces, np.int32).reshape(-1, 3) - 1, np.array(tets, np.int32).reshape(-1, 4) - 1
