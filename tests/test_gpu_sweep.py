"""The surrogate-steered sweep end to end on a small sweep: points run to
the end reproduce the plain sweep exactly (systems are independent and
deterministic), the surrogate saves particle-steps over the method without
it, and its answers on retired points stay near the full runs."""
import numpy as np
import pytest

from spp_gb300 import configs, surrogate

pytestmark = pytest.mark.gpu


def test_sweep_with_and_without_surrogate(gpu_lib):
    # the 512-point protocol with N in [256, 1024] and 4000 steps per point
    pts = configs.sweep_points(n_points=512, n_min=256, n_max=1024, seed=4)
    kw = dict(max_steps=4000, window=500, seed=4, chunk=1000)
    plain = surrogate.run_sweep(pts, use_surrogate=False, **kw)
    assert np.all(np.isfinite(plain.p_full))
    assert plain.particle_steps == plain.particle_steps_plain
    res = surrogate.run_sweep(pts, tol=0.02, **kw)
    ran = np.isfinite(res.p_full)
    # every point that ran to the end equals its plain run bit for bit
    assert np.array_equal(res.p_full[ran], plain.p_full[ran])
    assert not np.any(ran & res.retired) and np.all(ran | res.retired)
    assert res.heldout.sum() >= 1 and np.all(np.isfinite(res.heldout_err))
    err = np.abs(res.p_answer - plain.p_full)
    print(f"retired {res.retired.sum()} of {len(pts)}, work {res.particle_steps / plain.particle_steps:.3f}, "
          f"rounds {res.rounds}, scales {np.round(res.scales, 2)}, "
          f"retired |dP| {np.sort(err[res.retired])}, held-out |dP| {np.sort(res.heldout_err)}")
    # what the surrogate buys: fewer particle-steps at the same answers
    assert res.retired.sum() >= 50
    assert res.particle_steps < 0.9 * plain.particle_steps
    assert np.all(res.bound[res.retired] <= 0.02)
    assert np.mean(err[res.retired] <= 0.02) >= 0.8
    assert np.median(err[res.retired]) <= 0.01


def test_surrogate_saves_wall_time_on_the_full_sweep(gpu_lib):
    """What the network gains in wall-clock time: the 512-point sweep (N
    log-uniform in [1024, 65536], 20,000 steps), batched with the surrogate
    against batched without it, in points per hour counting only the answers
    within |dP| <= 0.02 of the full runs (measured: about 1.15x)."""
    pts = configs.sweep_points(seed=4)
    plain = surrogate.run_sweep(pts, use_surrogate=False, seed=4)
    res = surrogate.run_sweep(pts, tol=0.02, seed=4)
    err = np.abs(res.p_answer - plain.p_full)
    within = err <= 0.02
    gain = (within.sum() / res.wall_s) / (len(pts) / plain.wall_s)
    print(f"wall {res.wall_s:.2f} s against {plain.wall_s:.2f} s, {within.sum()} of {len(pts)} within "
          f"tolerance, gain {gain:.3f}, retired {res.retired.sum()}")
    assert np.mean(within) >= 0.97
    assert np.mean(err[res.retired] <= 0.02) >= 0.9
    assert gain >= 1.05
