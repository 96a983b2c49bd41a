"""The sweep surrogate's device kernels (spp_gb300/csrc/mlp.cu) against the
FP64 oracle (oracle/mlp_oracle.py): forward outputs, gradients, Adam steps
and a training run."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from spp_gb300 import surrogate

pytestmark = pytest.mark.gpu


def data(B=96, seed=1):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((B, 7)).astype(np.float32)
    t = (0.5 + 0.3 * np.tanh(x[:, 0] - 0.5 * x[:, 1])).astype(np.float32)
    return x, t


def test_forward_and_gradient_match_fp64(gpu_lib):
    x, t = data()
    mlp = surrogate.Mlp(ensemble=5, seed=7)
    theta = mlp.params()
    y = mlp.predict(x)
    g, loss = mlp.grad(x, t)
    for e in range(5):
        ye, _ = M.forward(theta[e], x)
        assert np.max(np.abs(y[e] - ye)) < 1e-4
        le, ge = M.loss_grad(theta[e], x, t)
        assert abs(loss[e] - le) <= 1e-4 * max(le, 1e-3)
        rel = np.linalg.norm(g[e] - ge) / np.linalg.norm(ge)
        assert rel < 1e-3, rel
    mlp.close()


def test_adam_step_matches_fp64(gpu_lib):
    x, t = data()
    mlp = surrogate.Mlp(ensemble=2, seed=8)
    theta = mlp.params().astype(np.float64)
    g, _ = mlp.grad(x, t)
    mlp.train(x, t, iters=1, lr=1e-3)
    after = mlp.params().astype(np.float64)
    for e in range(2):
        ref, _, _ = M.adam(theta[e], g[e].astype(np.float64), 0.0, 0.0, 1)
        assert np.max(np.abs(after[e] - ref)) < 1e-6
    mlp.close()


def test_training_reduces_loss_and_fits(gpu_lib):
    x, t = data(B=256)
    mlp = surrogate.Mlp(ensemble=5, seed=9)
    _, l0 = mlp.grad(x, t)
    l1 = mlp.train(x, t, iters=1500, lr=1e-3)
    assert np.all(l1 < 0.1 * l0)
    assert np.all(l1 < 1e-3)
    # the trained parameters still give the oracle's outputs
    theta = mlp.params()
    y = mlp.predict(x)
    ye, _ = M.forward(theta[0], x)
    assert np.max(np.abs(y[0] - ye)) < 1e-4
    mlp.close()


def test_weighted_gradient_matches_fp64(gpu_lib):
    """Per-member sample weights (K-fold bagging: zero weight leaves a sample
    out of that member's fit)."""
    x, t = data(B=40)
    mlp = surrogate.Mlp(ensemble=3, seed=11)
    theta = mlp.params()
    w = np.random.default_rng(3).uniform(0, 2, (3, 40)).astype(np.float32)
    w[1, ::4] = 0.0
    g, loss = mlp.grad(x, t, weights=w)
    for e in range(3):
        le, ge = M.loss_grad(theta[e], x, t, w[e])
        assert abs(loss[e] - le) <= 1e-4 * max(le, 1e-3)
        assert np.linalg.norm(g[e] - ge) / np.linalg.norm(ge) < 1e-3
    # a left-out sample does not move member 1's gradient
    t2 = t.copy()
    t2[0] += 5.0
    g2, _ = mlp.grad(x, t2, weights=w)
    assert np.array_equal(g2[1], g[1]) and not np.array_equal(g2[0], g[0])
    mlp.close()


def test_invalid_weights_are_rejected(gpu_lib):
    from spp_gb300 import abi
    x, t = data(B=8)
    mlp = surrogate.Mlp(ensemble=2, seed=1)
    w = np.ones((2, 8), np.float32)
    w[1] = 0.0
    with pytest.raises(abi.SppError):
        mlp.grad(x, t, weights=w)
    w[1] = -1.0
    with pytest.raises(abi.SppError):
        mlp.train(x, t, iters=1, weights=w)
    mlp.close()


def test_tensor_core_and_scalar_kernels_agree(gpu_lib, monkeypatch):
    """The 128 x 128 layer on the tensor cores (TF32 products of split FP32
    operands, FP32 sums) against the scalar FP32 kernels (SPP_MLP_SCALAR=1):
    outputs and gradients agree to FP32 rounding."""
    x, t = data(B=150)
    outs = []
    for scalar in ("0", "1"):
        monkeypatch.setenv("SPP_MLP_SCALAR", scalar)
        mlp = surrogate.Mlp(ensemble=3, seed=5)
        y = mlp.predict(x)
        g, loss = mlp.grad(x, t)
        outs.append((y, g, loss))
        mlp.close()
    (y0, g0, l0), (y1, g1, l1) = outs
    assert np.max(np.abs(y0 - y1)) < 1e-5
    for e in range(3):
        assert np.linalg.norm(g0[e] - g1[e]) / np.linalg.norm(g1[e]) < 1e-5
    assert np.allclose(l0, l1, rtol=1e-5)
