"""The FP64 surrogate oracle against finite differences (its gradient is
exact for the BF16-rounded weights), and the Philox initialisation."""
import numpy as np

from oracle import mlp_oracle as M
from spp_gb300 import surrogate


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    theta = surrogate.init_params(1, 7, seed=5)[0].astype(np.float64)
    x = rng.standard_normal((9, 7))
    t = rng.uniform(0, 1, 9)

    # finite differences on the float64 network (no BF16 rounding), so that
    # tiny perturbations are seen
    def loss(th):
        W1, b1, W2, b2, W3, b3 = M.unpack(th, 7)
        y = M.gelu(M.gelu(x @ W1.T + b1) @ W2.T + b2) @ W3 + b3
        return np.mean((y - t) ** 2)

    orig = M.bf16
    M.bf16 = lambda a: np.asarray(a, np.float64)
    try:
        _, g = M.loss_grad(theta, x, t)
    finally:
        M.bf16 = orig
    idx = rng.choice(len(theta), 40, replace=False)
    h = 1e-6
    for q in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[q] += h
        tm[q] -= h
        fd = (loss(tp) - loss(tm)) / (2 * h)
        assert abs(fd - g[q]) <= 1e-6 + 1e-4 * abs(fd)


def test_bf16_rounding_is_nearest_even():
    a = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], np.float32)
    b = M.bf16(a)
    assert b[0] == 1.0 and b[1] == 1.0  # tie at 1 + 2^-8 rounds to even
    assert b[2] == np.float32(1.0078125)
    assert b[3] == -2.5


def test_init_params_deterministic_and_scaled():
    a = surrogate.init_params(5, 7, seed=4)
    b = surrogate.init_params(5, 7, seed=4)
    assert np.array_equal(a, b) and a.shape == (5, surrogate.n_params(7))
    W1 = a[0, :128 * 7]
    assert np.abs(W1).max() <= 1 / np.sqrt(7) + 1e-6
    assert not np.array_equal(a[0], a[1])


def test_kfold_deals_every_fold():
    f = surrogate.kfold(23, 5, seed=4)
    assert np.array_equal(np.bincount(f), [5, 5, 5, 4, 4])
    assert np.array_equal(f, surrogate.kfold(23, 5, seed=4))


def test_oracle_weighted_loss_reduces_to_mean():
    rng = np.random.default_rng(2)
    theta = surrogate.init_params(1, 7, seed=5)[0]
    x = rng.standard_normal((12, 7))
    t = rng.uniform(0, 1, 12)
    l0, g0 = M.loss_grad(theta, x, t)
    l1, g1 = M.loss_grad(theta, x, t, np.full(12, 3.0))
    assert np.isclose(l0, l1) and np.allclose(g0, g1)
    w = np.ones(12)
    w[5] = 0
    l2, g2 = M.loss_grad(theta, np.delete(x, 5, 0), np.delete(t, 5))
    l3, g3 = M.loss_grad(theta, x, t, w)
    assert np.isclose(l2, l3) and np.allclose(g2, g3)
