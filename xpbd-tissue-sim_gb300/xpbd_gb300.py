"""Python binding of libxpbd_gpu.so (include/xpbd_gpu.h) through ctypes.

The product path is the CUDA library: there is no CPU fallback. Loading fails
loudly when the shared library is missing, and XPBDSolver raises when the C ABI
returns an error status.

Object model mirrors the reference's XPBDMeshObject_ + XPBDSolver surface:
  update()              XPBDMeshObject_::update        (src/simobject/XPBDMeshObject.cpp:426-505)
  velocity_update()     XPBDMeshObject_::velocityUpdate (XPBDMeshObject.cpp:507-535)
  step(n)               Simulation::_timeStep           (src/simulation/Simulation.cpp:197-276)
  fix_vertices(mask)    XPBDMeshObject_Base_::fixVertex (include/simobject/XPBDMeshObjectBase.hpp:97-99)
  constraint_residual() XPBDSolver::constraintResidual  (include/solver/xpbd_solver/XPBDSolver.hpp:135)
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_build", "libxpbd_gpu.so")
HEADER = os.path.join(ROOT, "include", "xpbd_gpu.h")

(XPBD_OK, XPBD_ERR_INVALID, XPBD_ERR_CUDA, XPBD_ERR_NUMERIC, XPBD_ERR_NO_DEVICE, XPBD_ERR_STATE, XPBD_ERR_CAPACITY,
 XPBD_ERR_TIMEOUT) = range(8)
SOLVER_GAUSS_SEIDEL, SOLVER_JACOBI = 0, 1
CONSTRAINT_COMBINED, CONSTRAINT_SEPARATE = 0, 1
RESIDUAL_NEVER, RESIDUAL_EVERY_SUBSTEP, RESIDUAL_EVERY_ITERATION = 0, 1, 2
JACOBI_ATOMIC, JACOBI_GATHER = 0, 1
WARM_NONE, WARM_PREVIOUS, WARM_MLP = 0, 1, 2
SDF_SPHERE, SDF_BOX, SDF_CYLINDER = 0, 1, 2
MLP_INPUTS, MLP_PARAMS = 16, 9538

# YAML `solver-type` strings (include/config/simobject/XPBDMeshObjectConfig.hpp:26-34)
# plus the GPU names; "Parallel-Jacobi" aliases the GPU Jacobi solver.
SOLVER_TYPES = {
    "Gauss-Seidel": SOLVER_GAUSS_SEIDEL,
    "GPU-Gauss-Seidel": SOLVER_GAUSS_SEIDEL,
    "Jacobi": SOLVER_JACOBI,
    "GPU-Jacobi": SOLVER_JACOBI,
    "Parallel-Jacobi": SOLVER_JACOBI,
}
CONSTRAINT_TYPES = {"Stable-Neohookean-Combined": CONSTRAINT_COMBINED, "Stable-Neohookean": CONSTRAINT_SEPARATE}
RESIDUAL_POLICIES = {"Never": RESIDUAL_NEVER, "Every-Substep": RESIDUAL_EVERY_SUBSTEP,
                     "Every-Iteration": RESIDUAL_EVERY_ITERATION}


class MeshDesc(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_int64), ("num_tets", C.c_int64), ("num_faces", C.c_int64),
        ("vertices", C.c_void_p), ("tets", C.c_void_p), ("faces", C.c_void_p),
        ("tet_E", C.c_void_p), ("tet_nu", C.c_void_p), ("tet_density", C.c_void_p),
    ]


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("g_accel", C.c_double), ("collision_rate", C.c_double),
        ("num_iters", C.c_int32), ("solver_type", C.c_int32), ("constraint_type", C.c_int32),
        ("residual_policy", C.c_int32), ("jacobi_variant", C.c_int32), ("block_size", C.c_int32),
        ("max_contacts_per_face", C.c_int32), ("use_graphs", C.c_int32), ("use_pdl", C.c_int32),
        ("gs_patch_tets", C.c_int32), ("gs_min_blocks", C.c_int32), ("gs_variant", C.c_int32),
        ("num_local_collision_iters", C.c_int32),
        ("first_order", C.c_int32), ("adjust_damping_to_material", C.c_int32), ("damping_multiplier", C.c_double),
        ("self_collisions", C.c_int32), ("gs_poll_ns", C.c_int32),
        ("gs_topology_reload", C.c_int32), ("gs_l2_stream", C.c_int32),
    ]


class XPBDError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"xpbd status {status}: {msg}")
        self.status = status


_lib = None


def header_functions() -> list[str]:
    """Names of the entry points include/xpbd_gpu.h declares."""
    import re
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"\b(xpbd_[a-z0-9_]+)\s*\(", text)


def load(path: str | None = None):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libxpbd_gpu.so not found at {path}: run __graft_entry__.build() "
                           f"(the solver has no CPU fallback)")
    L = C.CDLL(path)
    P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "xpbd_abi_version": ([], C.c_int),
        "xpbd_status_string": ([C.c_int], C.c_char_p),
        "xpbd_default_params": ([P], C.c_int),
        "xpbd_colour_items": ([I64, I32, P, I64, P], C.c_int),
        "xpbd_grid_counts": ([I32, I32, I32, P, P, P], C.c_int),
        "xpbd_grid_mesh": ([I32, I32, I32, D, D, D, I32, P, P, P], C.c_int),
        "xpbd_create": ([P, P, P], C.c_int),
        "xpbd_destroy": ([P], C.c_int),
        "xpbd_last_error": ([P], C.c_char_p),
        "xpbd_set_num_iters": ([P, I32], C.c_int),
        "xpbd_set_positions": ([P, P], C.c_int),
        "xpbd_get_positions": ([P, P], C.c_int),
        "xpbd_get_prev_positions": ([P, P], C.c_int),
        "xpbd_set_velocities": ([P, P], C.c_int),
        "xpbd_get_velocities": ([P, P], C.c_int),
        "xpbd_set_positions_f32": ([P, P], C.c_int),
        "xpbd_get_positions_f32": ([P, P], C.c_int),
        "xpbd_get_masses": ([P, P], C.c_int),
        "xpbd_set_fixed": ([P, P], C.c_int),
        "xpbd_set_kinematic_group": ([P, I32, P], C.c_int),
        "xpbd_set_kinematic_offset": ([P, P], C.c_int),
        "xpbd_set_spheres": ([P, I32, P, P], C.c_int),
        "xpbd_clear_collisions": ([P], C.c_int),
        "xpbd_detect_collisions": ([P], C.c_int),
        "xpbd_add_static_collision": ([P, I32, D, D, D, P, P], C.c_int),
        "xpbd_get_collisions": ([P, I32, P, P], C.c_int),
        "xpbd_update": ([P], C.c_int),
        "xpbd_solve": ([P], C.c_int),
        "xpbd_solve_local": ([P, I32], C.c_int),
        "xpbd_velocity_update": ([P], C.c_int),
        "xpbd_step": ([P, I32], C.c_int),
        "xpbd_synchronize": ([P], C.c_int),
        "xpbd_get_time": ([P, P], C.c_int),
        "xpbd_residual": ([P, P, P], C.c_int),
        "xpbd_get_constraint_residual": ([P, P, I64], C.c_int),
        "xpbd_residual_history": ([P, P, I32, P], C.c_int),
        "xpbd_get_lambda": ([P, P], C.c_int),
        "xpbd_total_strain_energy": ([P, P], C.c_int),
        "xpbd_health": ([P, P, P], C.c_int),
        "xpbd_debug_stall_vertex": ([P, I32, I32], C.c_int),
        "xpbd_num_colours": ([P, P, P], C.c_int),
        "xpbd_get_tet_colours": ([P, P], C.c_int),
        "xpbd_get_sweep_order": ([P, P], C.c_int),
        "xpbd_profile_steps": ([P, I32, I32, P, P], C.c_int),
        "xpbd_kernel_name": ([I32], C.c_char_p),
        "xpbd_launch_count": ([P, P], C.c_int),
        "xpbd_set_rigid_body": ([P, C.c_int32, C.c_int32, C.c_double, P, P, P], C.c_int),
        "xpbd_get_self_contacts": ([P, C.c_int32, P, P, P], C.c_int),
        "xpbd_get_rigid_body": ([P, C.c_int32, C.c_int32, P], C.c_int),
        "xpbd_get_stream": ([P, P], C.c_int),
        "xpbd_create_batch": ([P, I32, P, P], C.c_int),
        "xpbd_num_instances": ([P, P], C.c_int),
        "xpbd_instance_offsets": ([P, P, P, P], C.c_int),
        "xpbd_set_latency_stamps": ([P, I32], C.c_int),
        "xpbd_instance_latencies": ([P, P, P], C.c_int),
        "xpbd_set_instance_spheres": ([P, I32, I32, P, P], C.c_int),
        "xpbd_autotune": ([P, I32, P, I32, P, I32], C.c_int),
        "xpbd_mlp_init": ([P, C.c_uint64], C.c_int),
        "xpbd_mlp_set_params": ([P, P, I64], C.c_int),
        "xpbd_mlp_get_params": ([P, P, I64], C.c_int),
        "xpbd_mlp_forward": ([P, P, I64, P], C.c_int),
        "xpbd_mlp_loss_grad": ([P, P, P, I64, P, P], C.c_int),
        "xpbd_mlp_adam_step": ([P, P, C.c_float], C.c_int),
        "xpbd_mlp_record": ([P, I32], C.c_int),
        "xpbd_mlp_get_samples": ([P, P, P], C.c_int),
        "xpbd_mlp_train": ([P, I32, I32, C.c_float, P], C.c_int),
        "xpbd_set_warm_start": ([P, I32], C.c_int),
        "xpbd_warm_start_stats": ([P, P, P], C.c_int),
        "xpbd_residual_noalloc": ([P, P], C.c_int),
        "xpbd_get_local_order": ([P, P, P, I32, P], C.c_int),
        "xpbd_set_sdfs": ([P, I32, P, P, P, P], C.c_int),
        "xpbd_add_attachment": ([P, I32, P, P, P], C.c_int),
        "xpbd_set_attachment_point": ([P, I32, P], C.c_int),
        "xpbd_clear_attachments": ([P], C.c_int),
        "xpbd_num_attachments": ([P, P], C.c_int),
        "xpbd_set_instance_sdfs": ([P, I32, I32, P, P, P, P], C.c_int),
        "xpbd_sdf_eval": ([I32, P, P, P, I64, P, P], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_params(**kw) -> Params:
    p = Params()
    load().xpbd_default_params(C.byref(p))
    for k, v in kw.items():
        if k == "solver_type" and isinstance(v, str):
            v = SOLVER_TYPES[v]
        if k == "constraint_type" and isinstance(v, str):
            v = CONSTRAINT_TYPES[v]
        if k == "residual_policy" and isinstance(v, str):
            v = RESIDUAL_POLICIES[v]
        setattr(p, k, v)
    return p


def colour_items(items: np.ndarray, n_vertices: int):
    items = np.ascontiguousarray(items, np.int32)
    out = np.zeros(items.shape[0], np.int32)
    n = load().xpbd_colour_items(items.shape[0], items.shape[1], _p(items), n_vertices, _p(out))
    if n < 0:
        raise XPBDError(-n, "bad colouring input")
    return n, out


def grid_mesh(nx: int, ny: int, nz: int, hx: float, hy: float | None = None, hz: float | None = None,
              split: int = 0):
    """Hex grid with five tets per hex (createBeamMsh layout). Returns X (V,3),
    tets (T,4) int32, faces (F,3) int32."""
    hy = hx if hy is None else hy
    hz = hx if hz is None else hz
    L = load()
    nv, nt, nf = C.c_int64(), C.c_int64(), C.c_int64()
    st = L.xpbd_grid_counts(nx, ny, nz, C.byref(nv), C.byref(nt), C.byref(nf))
    if st != XPBD_OK:
        raise XPBDError(st, "bad grid size")
    X = np.zeros((nv.value, 3))
    tets = np.zeros((nt.value, 4), np.int32)
    faces = np.zeros((nf.value, 3), np.int32)
    st = L.xpbd_grid_mesh(nx, ny, nz, hx, hy, hz, split, _p(X), _p(tets), _p(faces))
    if st != XPBD_OK:
        raise XPBDError(st, "grid generation failed")
    return X, tets, faces


class _Mesh:
    """Host copies of one instance's arrays (kept alive for the C ABI call)."""

    def __init__(self, X, tets, faces, E, nu, density):
        self.X = np.ascontiguousarray(X, np.float64).reshape(-1, 3)
        self.tets = np.ascontiguousarray(tets, np.int32).reshape(-1, 4)
        self.faces = None if faces is None else np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
        T = self.tets.shape[0]
        bc = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), (T,)))
        self.E, self.nu, self.rho = bc(E), bc(nu), bc(density)

    def desc(self) -> MeshDesc:
        F = 0 if self.faces is None else self.faces.shape[0]
        return MeshDesc(self.X.shape[0], self.tets.shape[0], F, _p(self.X).value, _p(self.tets).value,
                        None if self.faces is None else _p(self.faces).value,
                        _p(self.E).value, _p(self.nu).value, _p(self.rho).value)


def autotune(instances, trial_steps=5, **params):
    """Times the candidate launch configurations on the given meshes
    (instances=[(X, tets, faces, E, nu, density), ...]) and returns
    (best Params, list of candidate results)."""
    import json
    L = load()
    meshes = [_Mesh(*inst) for inst in instances]
    descs = (MeshDesc * len(meshes))(*[m.desc() for m in meshes])
    p = default_params(**params)
    buf = C.create_string_buffer(1 << 16)
    st = L.xpbd_autotune(descs, len(meshes), C.byref(p), int(trial_steps), buf, len(buf))
    if st != XPBD_OK:
        raise XPBDError(st, L.xpbd_status_string(st).decode())
    return p, json.loads(buf.value.decode())


class XPBDSolver:
    """One deformable tet-mesh object solved on the GPU, or a batch of
    independent objects (instances=[(X, tets, faces, E, nu, density), ...])."""

    def __init__(self, X=None, tets=None, faces=None, E=3e3, nu=0.45, density=1000.0, instances=None, **params):
        self.L = load()
        meshes = [_Mesh(*inst) for inst in instances] if instances is not None else \
            [_Mesh(X, tets, faces, E, nu, density)]
        self.n_instances = len(meshes)
        self.V = sum(m.X.shape[0] for m in meshes)
        self.T = sum(m.tets.shape[0] for m in meshes)
        self.F = sum(0 if m.faces is None else m.faces.shape[0] for m in meshes)
        self.params = default_params(**params)
        descs = (MeshDesc * len(meshes))(*[m.desc() for m in meshes])
        h = C.c_void_p()
        st = self.L.xpbd_create_batch(descs, len(meshes), C.byref(self.params), C.byref(h))
        if st != XPBD_OK:
            raise XPBDError(st, self.L.xpbd_status_string(st).decode())
        self.h = h
        self._meshes = meshes

    # ---- lifetime ----
    def close(self):
        if getattr(self, "h", None):
            self.L.xpbd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        if st != XPBD_OK:
            raise XPBDError(st, self.L.xpbd_last_error(self.h).decode())

    # ---- state ----
    def positions(self, out=None) -> np.ndarray:
        """Current positions (V, 3) float64; into `out` (C-contiguous float64) when given."""
        if out is None:
            out = np.zeros((self.V, 3))
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.shape != (self.V, 3):
            raise ValueError("out must be a C-contiguous (V, 3) float64 array")
        self._ck(self.L.xpbd_get_positions(self.h, _p(out)))
        return out

    def prev_positions(self) -> np.ndarray:
        out = np.zeros((self.V, 3))
        self._ck(self.L.xpbd_get_prev_positions(self.h, _p(out)))
        return out

    def set_positions(self, x):
        x = np.ascontiguousarray(x, np.float64)
        self._ck(self.L.xpbd_set_positions(self.h, _p(x)))

    def velocities(self) -> np.ndarray:
        out = np.zeros((self.V, 3))
        self._ck(self.L.xpbd_get_velocities(self.h, _p(out)))
        return out

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, np.float64)
        self._ck(self.L.xpbd_set_velocities(self.h, _p(v)))

    def positions_f32(self, out=None) -> np.ndarray:
        out = np.zeros((self.V, 3), np.float32) if out is None else out
        self._ck(self.L.xpbd_get_positions_f32(self.h, _p(out)))
        return out

    def set_positions_f32(self, x):
        self._ck(self.L.xpbd_set_positions_f32(self.h, _p(np.ascontiguousarray(x, np.float32))))

    def masses(self) -> np.ndarray:
        out = np.zeros(self.V)
        self._ck(self.L.xpbd_get_masses(self.h, _p(out)))
        return out

    def fix_vertices(self, mask):
        m = np.ascontiguousarray(mask, np.uint8)
        self._ck(self.L.xpbd_set_fixed(self.h, _p(m)))

    def set_kinematic_group(self, idx):
        idx = np.ascontiguousarray(idx, np.int32)
        self._ck(self.L.xpbd_set_kinematic_group(self.h, len(idx), _p(idx)))

    def set_kinematic_offset(self, off):
        self._ck(self.L.xpbd_set_kinematic_offset(self.h, _p(np.ascontiguousarray(off, np.float64))))

    def set_num_iters(self, n):
        self._ck(self.L.xpbd_set_num_iters(self.h, int(n)))
        self.params.num_iters = int(n)

    # ---- collisions ----
    def set_spheres(self, centers, radii, instance=0):
        c = np.ascontiguousarray(centers, np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(radii, np.float64).reshape(-1)
        self._ck(self.L.xpbd_set_instance_spheres(self.h, int(instance), len(r), _p(c), _p(r)))

    def set_sdfs(self, kinds, positions, quats, dims, instance=0):
        """Fixed rigid primitives (SDF_SPHERE / SDF_BOX / SDF_CYLINDER) with
        orientation quaternions (x, y, z, w)."""
        k = np.ascontiguousarray(kinds, np.int32).reshape(-1)
        n = k.size
        p = np.ascontiguousarray(positions, np.float64).reshape(n, 3)
        q = np.ascontiguousarray(quats, np.float64).reshape(n, 4)
        d = np.ascontiguousarray(dims, np.float64).reshape(n, 3)
        self._ck(self.L.xpbd_set_instance_sdfs(self.h, int(instance), n, _p(k), _p(p), _p(q), _p(d)))

    def add_attachment(self, vertex, point, offset=(0.0, 0.0, 0.0)) -> int:
        p = np.ascontiguousarray(point, np.float64)
        o = np.ascontiguousarray(offset, np.float64)
        i = C.c_int32()
        self._ck(self.L.xpbd_add_attachment(self.h, int(vertex), _p(p), _p(o), C.byref(i)))
        return i.value

    def set_attachment_point(self, attachment, point):
        p = np.ascontiguousarray(point, np.float64)
        self._ck(self.L.xpbd_set_attachment_point(self.h, int(attachment), _p(p)))

    def clear_attachments(self):
        self._ck(self.L.xpbd_clear_attachments(self.h))

    def instance_offsets(self):
        """(vertex, tet, face) offsets of each instance, n + 1 entries each."""
        n = self.n_instances + 1
        v, t, f = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n, np.int64)
        self._ck(self.L.xpbd_instance_offsets(self.h, _p(v), _p(t), _p(f)))
        return v, t, f

    def set_latency_stamps(self, on: bool = True):
        """Stamp each substep's start and end and each persistent-sweep task's
        last iteration with the device clock (gs_variant 4 only)."""
        self._ck(self.L.xpbd_set_latency_stamps(self.h, int(bool(on))))

    def instance_latencies(self):
        """For the last stamped substep: (ms per instance from the substep's
        start to the end of that instance's last sweep task, ms of the whole
        substep)."""
        ms = np.zeros(self.n_instances, np.float64)
        b = C.c_double(0.0)
        self._ck(self.L.xpbd_instance_latencies(self.h, _p(ms), C.byref(b)))
        return ms, b.value

    def clear_collisions(self):
        self._ck(self.L.xpbd_clear_collisions(self.h))

    def detect_collisions(self):
        self._ck(self.L.xpbd_detect_collisions(self.h))

    def add_static_collision(self, face, u, v, w, p, n):
        self._ck(self.L.xpbd_add_static_collision(self.h, int(face), u, v, w,
                                                  _p(np.ascontiguousarray(p, np.float64)),
                                                  _p(np.ascontiguousarray(n, np.float64))))

    def collisions(self) -> np.ndarray:
        n = C.c_int32()
        self._ck(self.L.xpbd_get_collisions(self.h, 0, None, C.byref(n)))
        out = np.zeros((n.value, 12))
        if n.value:
            self._ck(self.L.xpbd_get_collisions(self.h, n.value, _p(out), C.byref(n)))
        return out

    # ---- stepping ----
    def update(self):
        self._ck(self.L.xpbd_update(self.h))

    def solve(self):
        """XPBDSolver::solve(): lambda <- 0 and num_iters sweeps on the current
        positions (no inertial move, no fixed reset)."""
        self._ck(self.L.xpbd_solve(self.h))

    def solve_local(self, num_iter):
        """XPBDSolver::solve(refs, num_iter, false) over the local collision set."""
        self._ck(self.L.xpbd_solve_local(self.h, int(num_iter)))

    def velocity_update(self):
        self._ck(self.L.xpbd_velocity_update(self.h))

    def step(self, n=1):
        self._ck(self.L.xpbd_step(self.h, int(n)))

    def synchronize(self):
        self._ck(self.L.xpbd_synchronize(self.h))

    @property
    def time(self) -> float:
        t = C.c_double()
        self._ck(self.L.xpbd_get_time(self.h, C.byref(t)))
        return t.value

    # ---- queries ----
    def residual(self):
        a, r = C.c_double(), C.c_double()
        self._ck(self.L.xpbd_residual(self.h, C.byref(a), C.byref(r)))
        return a.value, r.value

    def residual_history(self) -> np.ndarray:
        n = C.c_int32()
        buf = np.zeros(int(self.params.num_iters) + 2)
        self._ck(self.L.xpbd_residual_history(self.h, _p(buf), len(buf), C.byref(n)))
        return buf[: n.value].copy()

    def constraint_residual(self) -> np.ndarray:
        out = np.zeros(2 * self.T)
        self._ck(self.L.xpbd_get_constraint_residual(self.h, _p(out), out.size))
        return out

    def lambdas(self) -> np.ndarray:
        out = np.zeros((self.T, 2))
        self._ck(self.L.xpbd_get_lambda(self.h, _p(out)))
        return out

    def strain_energy(self) -> float:
        e = C.c_double()
        self._ck(self.L.xpbd_total_strain_energy(self.h, C.byref(e)))
        return e.value

    def health(self):
        a, b = C.c_int64(), C.c_int64()
        self._ck(self.L.xpbd_health(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def debug_stall_vertex(self, vertex: int, poll_limit: int = 0):
        """Test hook: the versioned sweep's waits on `vertex` never complete and
        give up after `poll_limit` polls (vertex < 0 restores the tables)."""
        self._ck(self.L.xpbd_debug_stall_vertex(self.h, int(vertex), int(poll_limit)))

    def colours(self):
        nt, nf = C.c_int32(), C.c_int32()
        self._ck(self.L.xpbd_num_colours(self.h, C.byref(nt), C.byref(nf)))
        col = np.zeros(self.T, np.int32)
        self._ck(self.L.xpbd_get_tet_colours(self.h, _p(col)))
        return nt.value, nf.value, col

    def sweep_order(self) -> np.ndarray:
        """Tets in the order one sweep projects them (Gauss-Seidel: colour by
        colour, patch by patch; Jacobi: index order)."""
        out = np.zeros(self.T, np.int32)
        self._ck(self.L.xpbd_get_sweep_order(self.h, _p(out)))
        return out

    def profile_steps(self, n):
        K = 16
        ms = np.zeros(K)
        cnt = np.zeros(K, np.int64)
        self._ck(self.L.xpbd_profile_steps(self.h, int(n), K, _p(ms), _p(cnt)))
        return {self.L.xpbd_kernel_name(k).decode(): (ms[k], int(cnt[k])) for k in range(K) if cnt[k]}

    def stream_handle(self) -> int:
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        h = C.c_void_p()
        self._ck(self.L.xpbd_get_stream(self.h, C.byref(h)))
        return h.value or 0

    def set_rigid_body(self, slot, mass, inertia, velocity=(0, 0, 0), angular_velocity=(0, 0, 0), instance=0):
        """SDF slot `slot` becomes a free rigid body (two-way coupling)."""
        a = [np.ascontiguousarray(v, np.float64).reshape(3) for v in (inertia, velocity, angular_velocity)]
        self._ck(self.L.xpbd_set_rigid_body(self.h, int(instance), int(slot), float(mass), _p(a[0]), _p(a[1]),
                                            _p(a[2])))

    def rigid_body(self, slot, instance=0):
        """(position, orientation (x, y, z, w), velocity, angular velocity) of a free body."""
        out = np.zeros(13)
        self._ck(self.L.xpbd_get_rigid_body(self.h, int(instance), int(slot), _p(out)))
        return out[:3], out[3:7], out[7:10], out[10:13]

    def self_contacts(self):
        """(rows of (surface vertex, face), multipliers) of the last detection."""
        n = C.c_int32()
        self._ck(self.L.xpbd_get_self_contacts(self.h, 0, None, None, C.byref(n)))
        vf = np.zeros((n.value, 2), np.int32)
        lam = np.zeros(n.value)
        if n.value:
            self._ck(self.L.xpbd_get_self_contacts(self.h, n.value, _p(vf), _p(lam), C.byref(n)))
        return vf, lam

    def launch_count(self) -> int:
        n = C.c_int64()
        self._ck(self.L.xpbd_launch_count(self.h, C.byref(n)))
        return n.value

    # ---- learned warm start ----
    def mlp_init(self, seed: int = 0):
        self._ck(self.L.xpbd_mlp_init(self.h, int(seed)))

    def mlp_params(self) -> np.ndarray:
        p = np.zeros(MLP_PARAMS, np.float32)
        self._ck(self.L.xpbd_mlp_get_params(self.h, _p(p), MLP_PARAMS))
        return p

    def set_mlp_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._ck(self.L.xpbd_mlp_set_params(self.h, _p(p), p.size))

    def mlp_forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32).reshape(-1, MLP_INPUTS)
        out = np.zeros((X.shape[0], 2), np.float32)
        self._ck(self.L.xpbd_mlp_forward(self.h, _p(X), X.shape[0], _p(out)))
        return out

    def mlp_loss_grad(self, X, Y):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, MLP_INPUTS)
        Y = np.ascontiguousarray(Y, np.float32).reshape(-1, 2)
        loss = C.c_double()
        g = np.zeros(MLP_PARAMS, np.float32)
        self._ck(self.L.xpbd_mlp_loss_grad(self.h, _p(X), _p(Y), X.shape[0], C.byref(loss), _p(g)))
        return loss.value, g

    def mlp_adam_step(self, lr: float = 1e-3, grad=None):
        g = None if grad is None else np.ascontiguousarray(grad, np.float32)
        self._ck(self.L.xpbd_mlp_adam_step(self.h, None if g is None else _p(g), float(lr)))

    def mlp_record(self, on: bool = True):
        self._ck(self.L.xpbd_mlp_record(self.h, 1 if on else 0))

    def mlp_samples(self):
        X = np.zeros((self.T, MLP_INPUTS), np.float32)
        Y = np.zeros((self.T, 2), np.float32)
        self._ck(self.L.xpbd_mlp_get_samples(self.h, _p(X), _p(Y)))
        return X, Y

    def mlp_train(self, epochs: int = 1, batch: int = 65536, lr: float = 1e-3) -> float:
        loss = C.c_double()
        self._ck(self.L.xpbd_mlp_train(self.h, int(epochs), int(batch), float(lr), C.byref(loss)))
        return loss.value

    def set_warm_start(self, mode: int):
        self._ck(self.L.xpbd_set_warm_start(self.h, int(mode)))

    def local_order(self):
        """(tet order, colour offsets) of the Gauss-Seidel local collision passes."""
        order = np.zeros(self.T, np.int32)
        off = np.zeros(1025, np.int32)
        n = C.c_int32()
        self._ck(self.L.xpbd_get_local_order(self.h, _p(order), _p(off), off.size, C.byref(n)))
        return order, off[: n.value + 1].copy()

    def residual_noalloc(self) -> float:
        """||r|| at the current state through the non-allocating entry point."""
        v = C.c_double()
        self._ck(self.L.xpbd_residual_noalloc(self.h, C.byref(v)))
        return v.value

    def warm_start_stats(self):
        k, r = C.c_int64(), C.c_int64()
        self._ck(self.L.xpbd_warm_start_stats(self.h, C.byref(k), C.byref(r)))
        return k.value, r.value


def sdf_eval(kind, position, quat, dims, points) -> np.ndarray:
    """(n, 4): SDF value and gradient of one primitive at points, on the GPU."""
    L = load()
    pos = np.ascontiguousarray(position, np.float64)
    q = np.ascontiguousarray(quat, np.float64)
    d = np.ascontiguousarray(dims, np.float64)
    pts = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
    out = np.zeros((pts.shape[0], 4))
    st = L.xpbd_sdf_eval(int(kind), _p(pos), _p(q), _p(d), pts.shape[0], _p(pts), _p(out))
    if st != XPBD_OK:
        raise XPBDError(st, "sdf_eval failed")
    return out
