"""Batched independent systems (sweep): each system of a batch must evolve
exactly as the same system run alone (its own Philox system id), and the
device-side polarization statistics must equal those computed from the
mirror's trajectory."""
import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import Batch, abi, configs

pytestmark = pytest.mark.gpu


def small_points(k=6, seed=9):
    pts = configs.sweep_points(n_points=k, n_min=300, n_max=3000, seed=seed)
    if k > 2:
        pts[2].model = abi.MODEL_VICSEK_REF_ANGLE
    if k > 3:
        pts[3].model = abi.MODEL_VICSEK_REF_VECTOR
    return pts


def split(arr, b):
    return [arr[b.offsets[s]:b.offsets[s + 1]] for s in range(b.n_sys)]


def test_batch_bitexact_vs_single_systems(gpu_lib):
    pts = small_points()
    x, y, th = configs.sweep_state(pts, seed=9)
    with Batch(pts) as b:
        b.upload(x, y, th)
        b.step(60)
        gx, gy, gth, gix, giy = b.download()
        st = b.poll()
    for s, p in enumerate(pts):
        sl = slice(b.offsets[s], b.offsets[s + 1])
        m = O.run32(p, O.State32(x[sl], y[sl], th[sl]), 60)
        assert np.array_equal(gx[sl], m.x) and np.array_equal(gy[sl], m.y), s
        assert np.array_equal(gth[sl], m.th) and np.array_equal(gix[sl], m.ix), s
        assert st[s].steps == 60


def polarization_series(p, x, y, th, steps):
    s = O.State32(x, y, th)
    P = []
    for t in range(steps):
        O.run32(p, s, 1, step0=t)
        c = np.cos(s.th.astype(np.float64)).sum()
        sn = np.sin(s.th.astype(np.float64)).sum()
        P.append(np.hypot(c, sn) / p.n)
    return np.array(P)


def test_batch_statistics(gpu_lib):
    pts = small_points(k=3)
    x, y, th = configs.sweep_state(pts, seed=9)
    W, S0, T = 25, 30, 50
    with Batch(pts) as b:
        b.set_windows(W, S0, T)
        b.upload(x, y, th)
        b.step(70)  # stops at T
        st = b.poll()
    for s, p in enumerate(pts):
        sl = slice(b.offsets[s], b.offsets[s + 1])
        P = polarization_series(p, x[sl], y[sl], th[sl], T)
        w = P[:W]
        m1, m2 = w.mean(), (w ** 2).mean()
        assert st[s].steps == T and st[s].active == 0
        # P from the kernels' (cos, sin) vs float64 cos/sin of the headings
        assert abs(st[s].p_mean - m1) < 1e-6
        assert abs(st[s].p_var - (m2 - m1 * m1)) < 1e-6
        assert st[s].stationary_steps == T - S0
        assert abs(st[s].p_stationary - P[S0:].mean()) < 1e-6


def test_batch_retire_freezes_a_system(gpu_lib):
    pts = small_points(k=4)
    x, y, th = configs.sweep_state(pts, seed=9)
    with Batch(pts) as b:
        b.upload(x, y, th)
        b.step(20)
        mid = b.download()
        b.retire([1])
        b.step(15)
        end = b.download()
        st = b.poll()
    sl = slice(b.offsets[1], b.offsets[2])
    assert np.array_equal(mid[0][sl], end[0][sl]) and st[1].steps == 20 and st[1].active == 0
    assert st[0].steps == 35 and st[2].steps == 35
    p = pts[2]
    s2 = slice(b.offsets[2], b.offsets[3])
    m = O.run32(p, O.State32(x[s2], y[s2], th[s2]), 35)
    assert np.array_equal(end[2][s2], m.th)


def test_retired_systems_leave_the_launch_space_and_resume_exactly(gpu_lib):
    """Retire and resume change the compact launch space (the particles and
    cells of the active systems); every system still evolves exactly as it
    would alone for the steps it was active."""
    pts = small_points(k=6)
    x, y, th = configs.sweep_state(pts, seed=9)
    with Batch(pts) as b:
        b.upload(x, y, th)
        b.step(10)
        b.retire([0, 2, 5])
        b.step(25)
        b.resume([0, 5])
        b.step(15)
        gx, gy, gth, gix, giy = b.download()
        st = b.poll()
        launches = b.kernel_launches()
    expect = {0: 25, 1: 50, 2: 10, 3: 50, 4: 50, 5: 25}
    for s, p in enumerate(pts):
        sl = slice(b.offsets[s], b.offsets[s + 1])
        assert st[s].steps == expect[s], s
        m = O.run32(p, O.State32(x[sl], y[sl], th[sl]), expect[s])
        assert np.array_equal(gx[sl], m.x) and np.array_equal(gth[sl], m.th), s
        assert np.array_equal(gix[sl], m.ix) and np.array_equal(giy[sl], m.iy), s
    assert launches > 0


def test_all_retired_batch_steps_nothing(gpu_lib):
    pts = small_points(k=3)
    x, y, th = configs.sweep_state(pts, seed=9)
    with Batch(pts) as b:
        b.upload(x, y, th)
        b.step(5)
        b.retire([0, 1, 2])
        b.step(7)
        st = b.poll()
        gx = b.download()[0]
    assert [q.steps for q in st] == [5, 5, 5]
    for s, p in enumerate(pts):
        sl = slice(b.offsets[s], b.offsets[s + 1])
        m = O.run32(p, O.State32(x[sl], y[sl], th[sl]), 5)
        assert np.array_equal(gx[sl], m.x)
