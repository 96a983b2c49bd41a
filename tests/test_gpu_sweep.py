"""The surrogate-steered sweep end to end on a small sweep: points run to
the end reproduce the plain sweep exactly (systems are independent and
deterministic), retired points are answered within the accuracy bar, and the
surrogate saves particle-steps over the method without it."""
import numpy as np
import pytest

from spp_gb300 import configs, surrogate

pytestmark = pytest.mark.gpu


def small_sweep():
    return configs.sweep_points(n_points=60, n_min=400, n_max=1600, rho=(0.5, 2.0), seed=21)


def test_sweep_with_and_without_surrogate(gpu_lib):
    pts = small_sweep()
    kw = dict(max_steps=1600, window=200, seed=21, chunk=400)
    plain = surrogate.run_sweep(pts, use_surrogate=False, **kw)
    assert np.all(np.isfinite(plain.p_full))
    res = surrogate.run_sweep(pts, spread_threshold=0.03, **kw)
    ran = np.isfinite(res.p_full)
    # every point that ran to the end equals its plain run bit for bit
    assert np.array_equal(res.p_full[ran], plain.p_full[ran])
    # the judge: held-out points compared with their full runs
    assert res.heldout.sum() >= 1 and np.all(np.isfinite(res.heldout_err))
    # what the surrogate buys: fewer particle-steps
    print("retired", res.retired.sum(), "of", len(pts), "work", res.particle_steps / plain.particle_steps,
          "held-out |dP| mean", res.heldout_err.mean(), "retired |dP| mean",
          np.abs(res.p_answer[res.retired] - plain.p_full[res.retired]).mean() if res.retired.any() else 0)
    assert res.particle_steps < plain.particle_steps
    if res.retired.any():
        err = np.abs(res.p_answer[res.retired] - plain.p_full[res.retired])
        assert err.mean() < 0.05
