"""The launch-shape autotuner on the device.

- The Verlet skin is a pure performance choice: trajectories with skins of
  0.3, 0.45 and 0.6 are bit-identical (every list is summed in particle-id
  order), for one lane and for four.
- gather_lanes named explicitly (four lanes above the automatic 16,384
  limit, one lane below it) stays bit-exact against the CPU mirror.
- spp_autotune times its eight candidates, chooses the fastest clean one,
  and the tuned system is bit-exact against the mirror; tuned_params fills
  its table once and then answers from it.
"""
import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import System, abi, autotune, configs

pytestmark = pytest.mark.gpu


def run_gpu(p, x, y, th, steps):
    with System(p) as s:
        s.upload(x, y, th)
        s.step(steps)
        out = s.download()
        obs = s.observables()
    return out, obs


def assert_same(a, b):
    for name, u, v in zip(("x", "y", "theta", "img_x", "img_y"), a, b):
        bad = np.flatnonzero(u != v)
        assert bad.size == 0, f"{name}: {bad.size} particles differ, first {bad[:5]}"


def assert_mirror(gpu, ref):
    assert_same(gpu, (ref.x, ref.y, ref.th, ref.ix, ref.iy))


@pytest.mark.parametrize("lanes", [1, 4])
def test_skin_does_not_change_the_trajectory(gpu_lib, lanes):
    p = configs.abp_config(n=4096, L=32.0, seed=1).replace(gather_lanes=lanes)
    x, y, th = configs.random_state(p.n, p.L, seed=1)
    base, obs = run_gpu(p, x, y, th, 150)
    assert obs.late_rebuilds == 0
    rebuilds = {0.3: obs.n_rebuilds}
    for skin in (0.45, 0.6):
        other, o = run_gpu(p.replace(skin=skin), x, y, th, 150)
        assert_same(base, other)
        assert o.late_rebuilds == 0
        rebuilds[skin] = o.n_rebuilds
    assert rebuilds[0.3] >= rebuilds[0.45] >= rebuilds[0.6] and rebuilds[0.3] > rebuilds[0.6]


@pytest.mark.parametrize("n,L,lanes", [(20000, 70.7, 4), (4096, 32.0, 1)])
def test_explicit_lanes_bitexact_vs_mirror(gpu_lib, n, L, lanes):
    p = configs.abp_config(n=n, L=L, seed=2).replace(gather_lanes=lanes)
    x, y, th = configs.random_state(n, L, seed=2)
    gpu, _ = run_gpu(p, x, y, th, 40)
    assert_mirror(gpu, O.run32(p, O.State32(x, y, th), 40))


def test_autotune_chooses_the_fastest_candidate_and_stays_exact(gpu_lib, tmp_path):
    p = configs.abp_config(n=20000, L=70.7, seed=3)
    x, y, th = configs.random_state(p.n, p.L, seed=3)
    q, rows = autotune.autotune(p, x, y, th, trial_steps=100)
    assert len(rows) == 8
    assert {(r["gather_lanes"], round(r["skin"] / p.skin, 3)) for r in rows} == \
        {(a, f) for a in (1, 4) for f in (0.5, 1.0, 1.5, 2.0)}
    clean = [r for r in rows if r["status"] == 0 and r["late_rebuilds"] == 0]
    assert clean and all(r["ms_per_step"] > 0 for r in clean)
    best = min(clean, key=lambda r: r["ms_per_step"])
    chosen = [r for r in rows if r["chosen"]]
    assert len(chosen) == 1 and chosen[0]["ms_per_step"] == best["ms_per_step"]
    assert (q.gather_lanes, q.skin) == (chosen[0]["gather_lanes"], chosen[0]["skin"])
    gpu, _ = run_gpu(q, x, y, th, 30)
    assert_mirror(gpu, O.run32(q, O.State32(x, y, th), 30))

    table = autotune.TuneTable(tmp_path / "tune.json")
    t1 = autotune.tuned_params(p, table=table, trial_steps=50)
    assert len(table.entries) == 1
    t2 = autotune.tuned_params(p, table=autotune.TuneTable(tmp_path / "tune.json"),
                               measure=lambda *a, **k: pytest.fail("measured again"))
    assert (t1.gather_lanes, t1.skin) == (t2.gather_lanes, t2.skin)
