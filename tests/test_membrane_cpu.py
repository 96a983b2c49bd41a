"""Ring membranes on the CPU: the bending and bond forces are the negative
gradient of E = k/2 sum (|b| - rest)^2 + kappa sum (1 - cos phi), and a
passive deformed ring relaxes (energy decreases, shape rounds)."""
import math

import numpy as np
import pytest

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


def _rtp(integ):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden import rtp_case
    return rtp_case(integ)


@pytest.mark.parametrize("integ", [abi.INT_EULER, abi.INT_RK2, abi.INT_RK4])
def test_mirror_tumbles_like_fp64(integ):
    """Run and tumble: the kernels' integer schedule (a start threshold on
    the 24-bit uniform, a tumble length counted in steps) makes the same
    decisions as the reference's double-precision rule, so the FP32 mirror
    stays within FP32 rounding of the FP64 restatement; one differing
    decision would cost a whole tumble step of turning (>= 0.006 rad here)."""
    p, x, y, th = _rtp(integ)
    th0 = th.copy()
    s32 = O.State32(x, y, th)
    O.run32(p, s32, 300)
    a = O.State64(x.copy(), y.copy(), th.copy())
    O.run64(p, a, 300)
    nb = p.n_rings * p.ring_size
    d = np.abs(((s32.th[nb:].astype(np.float64) - a.th[nb:]) + np.pi) % (2 * np.pi) - np.pi)
    assert d.max() < 1e-4
    assert np.abs(a.th[nb:] - th0[nb:]).max() > 0.1


def test_tumble_schedule_constants():
    """The step count of a tumble replays the reference's accumulation of dt
    in double (tumble_elapesed_time, particle.h:1092-1100)."""
    p, _, _, _ = _rtp(abi.INT_RK2)
    for t_tumble, dt in ((0.03, 0.002), (1.0, 0.1), (0.0, 0.01), (0.3, 0.1)):
        e, c = 0.0, 0
        while e < t_tumble:
            e += dt
            c += 1
        q = p.copy()
        q.tumble_time, q.dt = t_tumble, dt
        assert O.tumble_steps(q) == c


def _chains(integ, n=144):
    p = configs.chain_config(n=n, chain_beads=3, integrator=integ, seed=5, spacing=1.7)
    p.torque0 = 0.3
    x, y, th = configs.chain_state(p)
    return p, x, y, th


@pytest.mark.parametrize("integ", [abi.INT_EULER, abi.INT_RK2, abi.INT_RK4])
def test_mirror_tracks_fp64_chains(integ):
    """Interacting chiral trimers: the FP32 kernel arithmetic stays within
    FP32 rounding of the FP64 restatement of ActiveBrownianChain."""
    p, x, y, th = _chains(integ)
    s32 = O.State32(x, y, th)
    O.run32(p, s32, 200)
    a = O.State64(x.astype(np.float64), y.astype(np.float64), th.astype(np.float64))
    O.run64(p, a, 200)
    xu = s32.x.astype(np.float64) + 2 * p.L * s32.ix
    yu = s32.y.astype(np.float64) + 2 * p.L * s32.iy
    assert np.abs(xu - a.xu).max() < 1e-4 and np.abs(yu - a.yu).max() < 1e-4
    d = np.abs(((s32.th.astype(np.float64) - a.th) + np.pi) % (2 * np.pi) - np.pi)
    assert d.max() < 1e-3
    # the chains did interact: without forces the paths differ
    q = p.copy()
    q.force_law = abi.FORCE_NONE
    b = O.State64(x.astype(np.float64), y.astype(np.float64), th.astype(np.float64))
    O.run64(q, b, 200)
    assert np.hypot(a.xu - b.xu, a.yu - b.yu).max() > 1e-2


def test_free_chain_speed_and_turn_rate():
    """Without noise or neighbours a chain swims at v0 = m_parallel F0 along
    its heading and turns at k_perpendicular torque0 (Set_R0: the circle of
    radius R0 = v0 / (k torque0))."""
    p, x, y, th = _chains(abi.INT_RK4, n=16)
    p.force_law, p.Dr, p.torque0 = abi.FORCE_NONE, 0.0, 0.25
    ar = 1 / ((p.bead_separation * 2 / p.sigma_chain) + 1)
    k_perp = 6 / (1 + ar * ar) / p.sigma_chain ** 2   # Set_nb, particle.h:874
    s = O.State64(x.astype(np.float64), y.astype(np.float64), th.astype(np.float64))
    th0, x0, y0 = s.th.copy(), s.xu.copy(), s.yu.copy()
    steps = 500
    O.run64(p, s, steps)
    T = steps * p.dt
    w = k_perp * p.torque0
    off = ((s.th - th0 - w * T) + np.pi) % (2 * np.pi) - np.pi
    assert np.abs(off).max() < 1e-9
    # chord of the circle of radius v0 / w
    chord = np.hypot(s.xu - x0, s.yu - y0)
    assert np.abs(chord - 2 * p.v0 / w * np.sin(w * T / 2)).max() < 1e-9
