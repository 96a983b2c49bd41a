"""Lyapunov spectrum on the CPU: the linearised (tangent) estimator in FP32
with FP64 renormalisation (the kernels' arithmetic, via the mirror) and in
FP64 against the reference's own method, finite perturbations of the full
dynamics renormalised by Gram-Schmidt (parallel/lyapunovbox.h:128-194,
restated in oracle/spp_oracle64.c)."""
import numpy as np

from oracle import oracle as O
from spp_gb300 import configs


def setup(n=1024, K=4):
    p = configs.lyapunov_config(n=n)
    x, y, th = configs.random_state(p.n, p.L, seed=3)
    V = O.lyap_init32(p, K, 3)
    return p, x, y, th, V


def test_initial_vectors_orthonormal():
    p, x, y, th, V = setup()
    M = V.reshape(4, -1).astype(np.float64)
    assert np.allclose(M @ M.T, np.eye(4), atol=1e-6)


def test_tangent_estimators_agree_with_clone_method():
    p, x, y, th, V = setup()
    steps, m = 400, 10
    T = steps * p.dt
    V64 = V.astype(np.float64)
    ls32 = O.lyap_run32(p, O.State32(x, y, th), V.copy(), steps, m)
    ls64 = O.lyap_tangent64(p, O.State64(x, y, th), V64.copy(), steps, m)
    lsc = O.lyap_clone64(p, O.State64(x, y, th), V64.copy(), steps // m, m, 1e-7)
    lam32, lam64, lamc = ls32 / T, ls64 / T, lsc / T
    # the spec bar: within 2% of the FP64 run
    assert np.all(np.abs(lam32 - lam64) <= 0.02 * np.abs(lam64) + 1e-6)
    # linearisation vs finite 1e-7 perturbations of the reference's method
    assert np.all(np.abs(lam64 - lamc) <= 1e-3 * np.abs(lamc) + 1e-6)


def test_renormalisation_keeps_vectors_orthonormal():
    p, x, y, th, V = setup(K=3)
    O.lyap_run32(p, O.State32(x, y, th), V, 50, 7)
    M = V.reshape(3, -1).astype(np.float64)
    assert np.allclose(M @ M.T, np.eye(3), atol=1e-5)
