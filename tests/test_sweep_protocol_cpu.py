"""The host logic of the surrogate-steered sweep (spp_gb300.surrogate.run_sweep)
on the CPU, with the device batch and the device network replaced by small
numpy stand-ins: which points run to the end, which retire, how the first
conformal multiplier comes from the held-out points, and what the phase
record holds.  The GPU tests run the same protocol on the real kernels."""
import types

import numpy as np
import pytest

from spp_gb300 import configs, surrogate

MAX_STEPS, WINDOW = 400, 50


def truth_of(points):
    """A smooth stationary polarization per point (ordered at low noise)."""
    eta = np.array([p.eta for p in points])
    rho = np.array([p.n / (4.0 * p.L * p.L) for p in points])
    return 1.0 / (1.0 + np.exp(12.0 * (eta - 0.2 - 0.1 * rho)))


class FakeBatch:
    """Systems that advance in lockstep while active and stop at max_steps;
    the window moments are the truth plus seeded noise."""

    def __init__(self, points):
        self.n = len(points)
        self.truth = truth_of(points)
        rng = np.random.default_rng(7)
        self.w_mean = self.truth + 0.05 * rng.standard_normal(self.n)
        self.w_var = 0.01 + 0.02 * rng.random(self.n)
        self.w_kurt = 2.0 + rng.random(self.n)
        self.steps = np.zeros(self.n, np.int64)
        self.active = np.ones(self.n, bool)
        self.max_steps = None
        self.step_calls = 0

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def set_windows(self, window, stationary_from, max_steps):
        self.max_steps = max_steps

    def upload(self, x, y, th):
        pass

    def step(self, k):
        self.step_calls += 1
        a = self.active
        self.steps[a] = np.minimum(self.steps[a] + k, self.max_steps)
        self.active &= self.steps < self.max_steps

    def poll(self):
        return [types.SimpleNamespace(active=bool(self.active[s]), steps=int(self.steps[s]),
                                      p_stationary=float(self.truth[s]) if self.steps[s] >= self.max_steps else 0.0,
                                      p_mean=float(self.w_mean[s]), p_var=float(self.w_var[s]),
                                      p_kurt=float(self.w_kurt[s]))
                for s in range(self.n)]

    def retire(self, systems):
        self.active[np.asarray(systems, np.int64)] = False

    def resume(self, systems):
        s = np.asarray(systems, np.int64)
        self.active[s] = self.steps[s] < self.max_steps


class FakeMlp:
    """An ensemble of weighted ridge regressions on (features, features^2),
    member e fitted with its own sample weights (the K-fold bagging)."""

    def __init__(self, ensemble=5, in_dim=7, seed=4):
        self.E, self.in_dim = ensemble, in_dim
        self.coef = None

    def set_params(self, theta):
        self.coef = None

    def _design(self, x):
        x = np.asarray(x, np.float64)
        return np.hstack([np.ones((len(x), 1)), x, x ** 2])

    def train(self, x, t, iters=2000, lr=1e-3, weights=None):
        A = self._design(x)
        t = np.asarray(t, np.float64)
        w = np.ones((self.E, len(t))) if weights is None else np.asarray(weights, np.float64)
        self.coef = []
        for e in range(self.E):
            W = w[e]
            M = A.T @ (A * W[:, None]) + 1e-2 * np.eye(A.shape[1])
            self.coef.append(np.linalg.solve(M, A.T @ (W * t)))
        return np.zeros(self.E, np.float32)

    def predict(self, x):
        A = self._design(x)
        return np.stack([A @ c for c in self.coef]).astype(np.float32)


class RecordingSurrogate(surrogate.Surrogate):
    """Keeps every (mean, spread) prediction in call order."""

    def predict(self, f):
        m, s = super().predict(f)
        if not hasattr(self, "history"):
            self.history = []
        self.history.append((m.copy(), s.copy()))
        return m, s


@pytest.fixture
def fakes(monkeypatch):
    made = []

    def make_batch(points):
        b = FakeBatch(points)
        made.append(b)
        return b

    monkeypatch.setattr(surrogate, "Batch", make_batch)
    monkeypatch.setattr(surrogate, "Mlp", FakeMlp)
    return made


def points(n=160):
    return configs.sweep_points(n_points=n, n_min=64, n_max=256, seed=4)


def state(pts):
    m = sum(p.n for p in pts)
    z = np.zeros(m, np.float32)
    return z, z, z


def test_plain_sweep_runs_every_point_to_the_end(fakes):
    pts = points()
    res = surrogate.run_sweep(pts, max_steps=MAX_STEPS, window=WINDOW, use_surrogate=False, x0=state(pts),
                              chunk=100)
    assert np.array_equal(res.p_full, truth_of(pts))
    assert not res.retired.any()
    assert res.particle_steps == res.particle_steps_plain
    assert len(res.timings["phases"]) == 1 and res.timings["phases"][0]["points"] == len(pts)


@pytest.mark.parametrize("first_scale", ["heldout", "oof"])
def test_surrogate_sweep_partitions_the_points(fakes, first_scale):
    pts = points()
    sur = RecordingSurrogate(seed=4, iters=10)
    res = surrogate.run_sweep(pts, max_steps=MAX_STEPS, window=WINDOW, x0=state(pts), chunk=100, tol=0.02,
                              surrogate=sur, first_scale=first_scale)
    ran = np.isfinite(res.p_full)
    # the stand-ins leave both kinds of points and at least one fallback round
    assert res.retired.any() and ran.any() and res.rounds >= 1
    # every point is answered once: by its full run or by the network
    assert np.all(ran ^ res.retired)
    assert np.all(ran[res.heldout]) and not np.any(res.retired[res.heldout])
    # full runs are the truth; retired points carried a bound within tol
    assert np.allclose(res.p_full[ran], truth_of(pts)[ran])
    assert np.all(res.bound[res.retired] <= 0.02)
    assert np.array_equal(res.p_answer[ran], res.p_full[ran])
    assert res.heldout_err.size == res.heldout.sum()
    # the first run phase is the pilot plus the held-out points; no phase after
    # the last fallback round
    phases = res.timings["phases"]
    assert 1 <= len(phases) <= 1 + 1 + 1
    assert phases[0]["points"] == int(round(0.2 * len(pts))) + int(round(0.1 * len(pts)))
    assert res.particle_steps <= res.particle_steps_plain
    assert res.rounds == len(res.scales)


def test_first_multiplier_comes_from_the_held_out_points(fakes):
    pts = points()
    sur = RecordingSurrogate(seed=4, iters=10)
    res = surrogate.run_sweep(pts, max_steps=MAX_STEPS, window=WINDOW, x0=state(pts), chunk=100, tol=0.02,
                              surrogate=sur, first_scale="heldout")
    assert res.scales, "no round was needed"
    mean0, spread0 = sur.history[0]
    h = res.heldout
    expect = np.quantile(np.abs(mean0[h] - truth_of(pts)[h]) / sur.floor(spread0[h]), sur.coverage)
    assert res.scales[0] == pytest.approx(float(expect), rel=1e-12)
    oof = surrogate.run_sweep(pts, max_steps=MAX_STEPS, window=WINDOW, x0=state(pts), chunk=100, tol=0.02,
                              surrogate=RecordingSurrogate(seed=4, iters=10), first_scale="oof")
    assert oof.scales and oof.scales[0] != res.scales[0]


def test_lower_coverage_retires_at_least_as_many(fakes):
    pts = points()
    kw = dict(max_steps=MAX_STEPS, window=WINDOW, x0=state(pts), chunk=100, tol=0.02)
    strict = surrogate.run_sweep(pts, surrogate=RecordingSurrogate(seed=4, iters=10, coverage=0.95), **kw)
    loose = surrogate.run_sweep(pts, surrogate=RecordingSurrogate(seed=4, iters=10, coverage=0.5), **kw)
    assert loose.retired.sum() >= strict.retired.sum()
