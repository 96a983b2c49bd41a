"""Ring membranes on the CPU: the bending and bond forces are the negative
gradient of E = k/2 sum (|b| - rest)^2 + kappa sum (1 - cos phi), and a
passive deformed ring relaxes (energy decreases, shape rounds)."""
import math

import numpy as np

from oracle import oracle as O
from spp_gb300 import abi, configs


def ring_energy(x, y, L, M, k, rest, kappa):
    def mi(d):
        return d - 2 * L * np.floor(d / (2 * L) + 0.5)
    bx = mi(np.roll(x, -1) - x)
    by = mi(np.roll(y, -1) - y)
    b = np.hypot(bx, by)
    e = 0.5 * k * np.sum((b - rest) ** 2)
    c = (bx * np.roll(bx, 1) + by * np.roll(by, 1)) / (b * np.roll(b, 1))
    return e + kappa * np.sum(1 - c)


def passive_ring(M=48, aspect=1.6, L=40.0):
    p = configs.vesicle_config(n_rings=1, ring_size=M, swimmers_per_ring=0, L=L)
    p.n = M
    p.Dr = 0.0
    p.force_law = abi.FORCE_NONE  # ring mechanics only
    R = 0.5 / math.sin(math.pi / M)
    a = 2 * math.pi * np.arange(M) / M
    x = (R * aspect * np.cos(a)).astype(np.float32)
    y = (R / aspect * np.sin(a)).astype(np.float32)
    return p, x, y, np.zeros(M, np.float32)


def test_forces_are_energy_gradient():
    """One Euler step with a tiny dt moves beads by mu * F * dt: compare F with
    a central-difference gradient of the ring energy."""
    p, x, y, th = passive_ring()
    p.integrator = abi.INT_EULER
    p.force_law = abi.FORCE_NONE
    p.dt = 1e-7
    s = O.run64(p, O.State64(x, y, th), 1)
    F = np.stack([(s.xu - x) / (p.mu * p.dt), (s.yu - y) / (p.mu * p.dt)], 1)
    xd, yd = x.astype(np.float64), y.astype(np.float64)
    h = 1e-6
    G = np.zeros_like(F)
    for i in range(0, len(x), 7):
        for ax in range(2):
            xp, yp, xm, ym = xd.copy(), yd.copy(), xd.copy(), yd.copy()
            if ax == 0:
                xp[i] += h; xm[i] -= h
            else:
                yp[i] += h; ym[i] -= h
            ep = ring_energy(xp, yp, p.L, p.ring_size, p.k_bond, p.bond_rest, p.kappa_bend)
            em = ring_energy(xm, ym, p.L, p.ring_size, p.k_bond, p.bond_rest, p.kappa_bend)
            G[i, ax] = -(ep - em) / (2 * h)
    idx = np.arange(0, len(x), 7)
    assert np.allclose(F[idx], G[idx], rtol=1e-4, atol=1e-4)


def test_passive_ring_relaxes():
    """Overdamped dynamics only dissipates: the ring energy falls, and the
    bending term slowly rounds the ellipse."""
    p, x, y, th = passive_ring()
    e0 = ring_energy(x.astype(np.float64), y.astype(np.float64), p.L, p.ring_size, p.k_bond,
                     p.bond_rest, p.kappa_bend)
    def roughness(s):
        r = np.hypot(s.xu - s.xu.mean(), s.yu - s.yu.mean())
        return r.std() / r.mean()

    s = O.run64(p, O.State64(x, y, th), 3000)
    e1 = ring_energy(s.x, s.y, p.L, p.ring_size, p.k_bond, p.bond_rest, p.kappa_bend)
    r1 = roughness(s)
    assert e1 < 0.05 * e0
    O.run64(p, s, 17000, step0=3000)  # advances s in place
    e2 = ring_energy(s.x, s.y, p.L, p.ring_size, p.k_bond, p.bond_rest, p.kappa_bend)
    assert e2 <= e1
    assert roughness(s) < 0.9 * r1


def test_mirror_tracks_fp64_vesicles():
    p = configs.vesicle_config(n_rings=4, ring_size=40, swimmers_per_ring=8, L=20.0)
    x, y, th = configs.vesicle_state(p)
    a = O.run64(p, O.State64(x, y, th), 100)
    m = O.run32(p, O.State32(x, y, th), 100)
    xu = m.x.astype(np.float64) + 2 * p.L * m.ix
    assert np.max(np.abs(xu - a.xu)) / (2 * p.L) < 1e-6
