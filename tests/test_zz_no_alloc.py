"""xpbd_residual_noalloc, the residual entry point that allocates nothing,
against xpbd_residual through the C ABI. The file name sorts last so that the
suite also exercises it after every other test has used the device."""
import numpy as np
import pytest

import xpbd_gb300 as G

pytestmark = pytest.mark.gpu


def _solver(n=6, **kw):
    X, tets, _ = G.grid_mesh(n, n, n, 1.0 / n)
    rng = np.random.default_rng(n)
    s = G.XPBDSolver(X, tets, None, 3e3, 0.45, 1000.0, dt=1e-3, num_iters=5, **kw)
    s.fix_vertices(X[:, 2] == 0)
    s.set_positions(X + rng.uniform(-1e-3, 1e-3, X.shape))
    return s


@pytest.mark.parametrize("solver", [G.SOLVER_GAUSS_SEIDEL, G.SOLVER_JACOBI])
def test_matches_xpbd_residual_on_consecutive_calls(lib, solver):
    s = _solver(solver_type=solver)
    s.step(5)
    for _ in range(2):
        a = s.residual_noalloc()
        b, _ = s.residual()
        assert a > 0 and a == pytest.approx(b, rel=1e-12, abs=0)
    s.step(3)
    a1 = s.residual_noalloc()
    a2 = s.residual_noalloc()
    b, _ = s.residual()
    assert a1 == a2 and a1 == pytest.approx(b, rel=1e-12, abs=0)
    s.close()


def test_contexts_called_in_turn_share_the_scratch(lib):
    s1, s2 = _solver(4), _solver(7)
    s1.step(2)
    s2.step(4)
    for _ in range(2):
        for s in (s1, s2):
            a = s.residual_noalloc()
            b, _ = s.residual()
            assert a == pytest.approx(b, rel=1e-12, abs=0)
    s1.close()
    s2.close()


def test_rejects_meshes_beyond_the_fixed_scratch(lib):
    # 48^3 hexes x 5 = 552,960 tets at block 32 need 17,280 partial sums (> 16,384)
    s = _solver(48, block_size=32)
    with pytest.raises(G.XPBDError) as e:
        s.residual_noalloc()
    assert e.value.status == G.XPBD_ERR_CAPACITY
    # the allocating entry point still serves it
    b, _ = s.residual()
    assert np.isfinite(b)
    s.close()


def test_repeated_calls_take_no_device_memory(lib):
    torch = pytest.importorskip("torch")
    s = _solver(8)
    s.step(2)
    s.residual_noalloc()  # resolves the scratch address on this device
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        s.residual_noalloc()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0
    s.close()
