"""CPU tests of the C ABI library: it loads, exports every entry point that
include/xpbd_gpu.h declares, and its host-only utilities and argument checks
work without a GPU (no compute calls)."""
import ctypes as C
import subprocess

import numpy as np
import pytest

import oracle as O
import xpbd_gb300 as G


def test_library_exports_every_declared_entry_point(lib):
    declared = set(G.header_functions())
    assert len(declared) >= 40
    out = subprocess.run(["nm", "-D", "--defined-only", G.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if " T " in ln}
    missing = declared - exported
    assert not missing, missing
    for name in declared:
        assert hasattr(lib, name)


def test_abi_version_and_status_strings(lib):
    assert lib.xpbd_abi_version() == 8
    assert lib.xpbd_status_string(0) == b"ok"
    assert b"invalid" in lib.xpbd_status_string(G.XPBD_ERR_INVALID)


def test_default_params_follow_reference_defaults(lib):
    p = G.default_params()
    assert p.dt == 1e-3 and p.g_accel == 9.81 and p.collision_rate == 100.0
    assert p.num_iters == 1 and p.solver_type == G.SOLVER_GAUSS_SEIDEL
    assert p.constraint_type == G.CONSTRAINT_COMBINED and p.residual_policy == G.RESIDUAL_NEVER
    q = G.default_params(solver_type="Parallel-Jacobi", residual_policy="Every-Substep")
    assert q.solver_type == G.SOLVER_JACOBI and q.residual_policy == G.RESIDUAL_EVERY_SUBSTEP


@pytest.mark.parametrize("dims", [(2, 2, 2), (4, 4, 4), (3, 5, 2), (10, 100, 10)])
@pytest.mark.parametrize("split", [0, 1])
def test_product_grid_generator_matches_oracle(lib, oracle_mod, dims, split):
    a = G.grid_mesh(*dims, 0.1, 0.2, 0.3, split=split)
    b = O.grid_mesh(*dims, 0.1, 0.2, 0.3, split=split)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_colouring_matches_oracle_and_is_valid(lib, oracle_mod):
    X, tets, faces = G.grid_mesh(6, 5, 4, 0.1)
    n1, c1 = G.colour_items(tets, len(X))
    n2, c2 = O.greedy_colour(tets, len(X))
    assert n1 == n2
    np.testing.assert_array_equal(c1, c2)
    nf, cf = G.colour_items(faces, len(X))
    for c in range(nf):
        v = faces[cf == c].ravel()
        assert len(np.unique(v)) == len(v)
    with pytest.raises(G.XPBDError):
        G.colour_items(tets + 10_000, len(X))


def _create(lib, X, tets, params):
    T = len(tets)
    E = np.full(T, 3e3); nu = np.full(T, 0.45); rho = np.full(T, 1e3)
    d = G.MeshDesc(len(X), T, 0, X.ctypes.data, tets.ctypes.data, None, E.ctypes.data, nu.ctypes.data,
                   rho.ctypes.data)
    h = C.c_void_p()
    return lib.xpbd_create(C.byref(d), C.byref(params), C.byref(h)), h


def test_create_rejects_bad_parameters_before_touching_a_device(lib):
    X, tets, _ = G.grid_mesh(2, 2, 2, 0.5)
    for field, value in [("dt", -1.0), ("num_iters", -2), ("solver_type", 7), ("block_size", 48),
                         ("max_contacts_per_face", 99), ("gs_poll_ns", -1), ("gs_topology_reload", 2),
                         ("gs_l2_stream", 2), ("gs_l2_stream", -2)]:
        p = G.default_params()
        setattr(p, field, value)
        st, h = _create(lib, X, tets, p)
        assert st == G.XPBD_ERR_INVALID and not h.value


def test_create_rejects_empty_meshes(lib):
    """A mesh without tets or without vertices is an invalid input, refused
    before a device is touched."""
    X, tets, _ = G.grid_mesh(1, 1, 1, 1.0)
    p = G.default_params()
    for Xe, te in [(X, tets[:0]), (X[:0], tets)]:
        st, h = _create(lib, np.ascontiguousarray(Xe), np.ascontiguousarray(te), p)
        assert st == G.XPBD_ERR_INVALID and not h.value


def test_create_without_gpu_reports_no_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    X, tets, _ = G.grid_mesh(2, 2, 2, 0.5)
    st, h = _create(lib, X, tets, G.default_params())
    assert st == G.XPBD_ERR_NO_DEVICE and not h.value
    with pytest.raises(G.XPBDError) as e:
        G.XPBDSolver(X, tets)
    assert e.value.status == G.XPBD_ERR_NO_DEVICE


def test_null_context_calls_are_rejected(lib):
    assert lib.xpbd_step(None, 1) == G.XPBD_ERR_INVALID
    assert lib.xpbd_update(None) == G.XPBD_ERR_INVALID
    assert lib.xpbd_destroy(None) == G.XPBD_ERR_INVALID
    assert lib.xpbd_last_error(None) == b"null context"
