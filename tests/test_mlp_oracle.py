"""CPU checks of the warm-start network's oracle (oracle/mlp_oracle.py): BF16
rounding, the analytic gradient against central differences of the plain
FP64 network, and Adam against its closed form on one step."""
import numpy as np

import mlp_oracle as M


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 0.0, np.inf], np.float32)
    r = M.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1) wins;
    # 1 + 3 * 2^-8 ties between 1 + 2^-7 and 1 + 2^-6: even is 1 + 2^-6
    np.testing.assert_array_equal(r, [1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -2.5, 0.0, np.inf])
    assert np.isnan(M.bf16(np.array([np.nan], np.float32)))[0]


def test_flatten_roundtrip_and_layout():
    p = M.init_params(3)
    v = M.flatten(p)
    assert v.size == 9538
    q = M.unflatten(v)
    for a, b in zip(p, q):
        np.testing.assert_array_equal(a, b)
    # padding input columns of W1 start at zero
    assert np.all(p[0][:, 14:] == 0)


def test_gradient_matches_central_differences():
    rng = np.random.default_rng(0)
    p = [a.astype(np.float64) for a in M.init_params(1)]
    p[7] = rng.standard_normal(2)  # nonzero output bias
    X = rng.standard_normal((12, 16))
    X[:, 14:] = 0
    Y = rng.standard_normal((12, 2))
    _, g = M.loss_and_grads(p, X, Y, rounding=False)
    eps = 1e-6
    for k, idx in [(0, (3, 5)), (1, (7,)), (2, (10, 20)), (3, (0,)), (4, (63, 1)), (5, (30,)), (6, (1, 40)),
                   (7, (1,))]:
        pp = [a.copy() for a in p]
        pm = [a.copy() for a in p]
        pp[k][idx] += eps
        pm[k][idx] -= eps
        lp, _ = M.loss_and_grads(pp, X, Y, rounding=False)
        lm, _ = M.loss_and_grads(pm, X, Y, rounding=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k][idx]) <= 1e-6 * max(1.0, abs(fd)), (k, idx, fd, g[k][idx])


def test_adam_first_step_is_signed_lr():
    p = [np.array([1.0, -2.0], np.float32)]
    g = [np.array([0.5, -3.0])]
    m = [np.zeros(2)]
    v = [np.zeros(2)]
    q, m1, v1 = M.adam_step(p, g, m, v, 1, lr=1e-2)
    # bias-corrected first step: -lr * g / (|g| + eps')
    np.testing.assert_allclose(q[0], [1.0 - 1e-2, -2.0 + 1e-2], rtol=0, atol=1e-7)
    np.testing.assert_allclose(m1[0], 0.1 * g[0])
    np.testing.assert_allclose(v1[0], 0.001 * g[0] ** 2)
