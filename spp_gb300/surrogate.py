"""Surrogate-steered parameter sweep.

The reference resolves a sweep by running every point to the end, one
realisation per MPI rank (serial/mpi-main.cpp:157-176).  Here all points run
as one device batch (``Batch``), and an ensemble MLP trained on the sweep's
own completed runs predicts each point's stationary polarization from its
parameters and the moments of its polarization over a short start-up
window.  Points whose ensemble agrees retire after the window; the others,
and a held-out 10% that judges the surrogate, run to the end.

Protocol (``run_sweep``):
  1. every point runs ``window`` steps (device-side moments of P);
  2. a pilot subset and the held-out points run to ``max_steps``; their
     stationary P (mean over the second half) are the training targets and
     the judge's ground truth;
  3. the ensemble is trained on the pilot points (device kernels, Adam);
  4. remaining points: ensemble mean -> answer if the ensemble spread is
     below ``spread_threshold``, otherwise the point runs to ``max_steps``
     (the plain full run is the fallback); the surrogate is retrained on
     the fallback runs before the answers are final;
  5. the held-out points compare the surrogate's prediction with their full
     runs (the judge of its error).
"""
import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi, configs
from .system import Batch

HIDDEN = 128
N_FEATURES = 7


def n_params(in_dim=N_FEATURES):
    return HIDDEN * in_dim + HIDDEN + HIDDEN * HIDDEN + HIDDEN + HIDDEN + 1


def init_params(ensemble, in_dim=N_FEATURES, seed=4):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases, from
    the Philox stream (member e uses system word e)."""
    P = n_params(in_dim)
    out = np.zeros((ensemble, P), np.float32)
    for e in range(ensemble):
        ids = np.arange(P, dtype=np.uint32)
        u = configs.u01_f32(configs.draw(seed, 100 + e, ids, 0, 8)[0]).astype(np.float64)
        w = 2 * u - 1
        th = np.zeros(P)
        o = 0
        th[o:o + HIDDEN * in_dim] = w[o:o + HIDDEN * in_dim] / math.sqrt(in_dim)
        o = HIDDEN * in_dim + HIDDEN
        th[o:o + HIDDEN * HIDDEN] = w[o:o + HIDDEN * HIDDEN] / math.sqrt(HIDDEN)
        o = HIDDEN * in_dim + HIDDEN + HIDDEN * HIDDEN + HIDDEN
        th[o:o + HIDDEN] = w[o:o + HIDDEN] / math.sqrt(HIDDEN)
        out[e] = th.astype(np.float32)
    return out


class Mlp:
    """Ensemble MLP on the device (spp_mlp_*)."""

    def __init__(self, ensemble=5, in_dim=N_FEATURES, seed=4):
        self._h = C.c_void_p()
        abi.check(abi.lib().spp_mlp_create(ensemble, in_dim, C.byref(self._h)), "spp_mlp_create")
        self.E, self.in_dim = ensemble, in_dim
        self.P = abi.lib().spp_mlp_num_params(self._h)
        self.set_params(init_params(ensemble, in_dim, seed))

    def close(self):
        if self._h:
            abi.lib().spp_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, theta):
        theta = np.ascontiguousarray(theta, np.float32).reshape(self.E, self.P)
        abi.check(abi.lib().spp_mlp_set_params(self._h, abi.fptr(theta)), "spp_mlp_set_params")

    def params(self):
        out = np.empty((self.E, self.P), np.float32)
        abi.check(abi.lib().spp_mlp_get_params(self._h, abi.fptr(out)), "spp_mlp_get_params")
        return out

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        B = x.shape[0]
        y = np.empty((self.E, B), np.float32)
        abi.check(abi.lib().spp_mlp_predict(self._h, abi.fptr(x), B, abi.fptr(y)), "spp_mlp_predict")
        return y

    def grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.empty((self.E, self.P), np.float32)
        loss = np.empty(self.E, np.float32)
        abi.check(abi.lib().spp_mlp_grad(self._h, abi.fptr(x), abi.fptr(t), x.shape[0], abi.fptr(g),
                                         abi.fptr(loss)), "spp_mlp_grad")
        return g, loss

    def train(self, x, t, iters=2000, lr=1e-3):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = np.empty(self.E, np.float32)
        abi.check(abi.lib().spp_mlp_train(self._h, abi.fptr(x), abi.fptr(t), x.shape[0], int(iters),
                                          float(lr), abi.fptr(loss)), "spp_mlp_train")
        return loss


def raw_features(points, stats):
    """(eta, rho, v0, log N, mean P, var P, kurtosis P) per point."""
    f = np.zeros((len(points), N_FEATURES))
    for s, (p, st) in enumerate(zip(points, stats)):
        rho = p.n / (4.0 * p.L * p.L)
        f[s] = [p.eta, rho, p.v0, math.log(p.n), st.p_mean, st.p_var, st.p_kurt]
    return f


@dataclass
class Surrogate:
    ensemble: int = 5
    seed: int = 4
    iters: int = 3000
    lr: float = 1e-3
    mu: np.ndarray = field(default=None)
    sd: np.ndarray = field(default=None)
    mlp: Mlp = field(default=None)

    def _norm(self, f):
        return ((f - self.mu) / self.sd).astype(np.float32)

    def fit(self, f, target):
        self.mu = f.mean(0)
        self.sd = f.std(0) + 1e-9
        if self.mlp is None:
            self.mlp = Mlp(self.ensemble, f.shape[1], self.seed)
        else:
            self.mlp.set_params(init_params(self.ensemble, f.shape[1], self.seed))
        return self.mlp.train(self._norm(f), np.asarray(target, np.float32), self.iters, self.lr)

    def predict(self, f):
        y = self.mlp.predict(self._norm(f)).astype(np.float64)
        return y.mean(0), y.std(0)


@dataclass
class SweepResult:
    p_answer: np.ndarray          # stationary P reported per point
    p_full: np.ndarray            # P of the points run to the end (NaN otherwise)
    retired: np.ndarray           # bool: answered by the surrogate
    heldout: np.ndarray           # bool: judge points
    heldout_err: np.ndarray       # |prediction - full run| on the judge points
    particle_steps: int           # work actually done
    particle_steps_plain: int     # work of running every point to the end
    wall_s: float
    timings: dict


def run_sweep(points, max_steps=20000, window=500, pilot_frac=0.3, holdout_frac=0.1,
              spread_threshold=0.01, surrogate=None, seed=4, x0=None, use_surrogate=True,
              chunk=2000):
    """Runs the sweep described in the module docstring and returns a
    SweepResult.  With use_surrogate=False every point runs to the end (the
    plain batched sweep)."""
    t_start = time.perf_counter()
    timings = {}
    n = len(points)
    rng = np.random.default_rng(seed)
    order = rng.permutation(n)
    n_hold = max(1, int(round(holdout_frac * n)))
    heldout = np.zeros(n, bool)
    heldout[order[:n_hold]] = True
    pilot = np.zeros(n, bool)
    n_pilot = max(2, int(round(pilot_frac * n)))
    pilot[order[n_hold:n_hold + n_pilot]] = True
    stationary_from = max_steps // 2
    x, y, th = x0 if x0 is not None else configs.sweep_state(points, seed=seed)
    sizes = np.array([p.n for p in points], np.int64)
    with Batch(points) as b:
        b.set_windows(window, stationary_from, max_steps)
        b.upload(x, y, th)
        t0 = time.perf_counter()
        if use_surrogate:
            b.step(window)
            st = b.poll()
            f = raw_features(points, st)
            # only the pilot and held-out points continue for now
            b.retire(np.flatnonzero(~(pilot | heldout)))
        run_until_done(b, chunk)
        st = b.poll()
        timings["runs_s"] = time.perf_counter() - t0
        p_full = np.array([s.p_stationary if s.steps >= max_steps else np.nan for s in st])
        steps = np.array([s.steps for s in st], np.int64)
        retired = np.zeros(n, bool)
        p_answer = p_full.copy()
        heldout_err = np.array([])
        if use_surrogate:
            t1 = time.perf_counter()
            sur = surrogate or Surrogate(seed=seed)
            sur.fit(f[pilot], p_full[pilot])
            rest = ~(pilot | heldout)
            mean, spread = sur.predict(f)
            confident = rest & (spread <= spread_threshold)
            fallback = rest & ~confident
            timings["train_s"] = time.perf_counter() - t1
            # fallback points resume and run to the end
            if fallback.any():
                resume(b, np.flatnonzero(fallback))
                t2 = time.perf_counter()
                run_until_done(b, chunk)
                timings["fallback_runs_s"] = time.perf_counter() - t2
                st = b.poll()
                for s in np.flatnonzero(fallback):
                    p_full[s] = st[s].p_stationary
                    steps[s] = st[s].steps
                # retrain on everything that ran to the end before answering
                done = pilot | fallback
                sur.fit(f[done], p_full[done])
                mean, spread = sur.predict(f)
            retired = confident
            p_answer = np.where(confident, mean, p_full)
            heldout_err = np.abs(mean[heldout] - p_full[heldout])
        wall = time.perf_counter() - t_start
    return SweepResult(p_answer=p_answer, p_full=p_full, retired=retired, heldout=heldout,
                       heldout_err=heldout_err, particle_steps=int(np.sum(sizes * steps)),
                       particle_steps_plain=int(np.sum(sizes) * max_steps), wall_s=wall,
                       timings=timings)


def run_until_done(b, chunk):
    while True:
        st = b.poll()
        if not any(s.active for s in st):
            return
        b.step(chunk)


def resume(b, systems):
    idx = np.ascontiguousarray(systems, np.int32)
    abi.check(abi.lib().spp_batch_resume(b._h, abi.iptr(idx), len(idx)), "spp_batch_resume")
