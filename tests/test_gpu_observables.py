"""Device observables against the FP32 mirror (bit-exact counts) and against
per-step readouts: the radial and body-frame pair histograms of a state,
the recorded polarization series, and the batch's stationary Binder
cumulants."""
import numpy as np
import pytest

from oracle import analysis_oracle as A
from oracle import oracle as O
from spp_gb300 import SppError, Batch, System, configs, observables

pytestmark = pytest.mark.gpu


def vicsek_system(n=4096, L=32.0, eta=0.3, seed=0):
    p = configs.vicsek_config(n=n, L=L, eta=eta, seed=seed)
    x, y, th = configs.random_state(n, L, seed=seed)
    return p, x, y, th


def test_pair_histograms_bitexact_vs_mirror(gpu_lib):
    p, x, y, th = vicsek_system()
    with System(p) as s:
        s.upload(x, y, th)
        s.step(40)
        gx, gy, gth, _, _ = s.download()
        rad = s.radial_distribution(5.0, 50)
        pd = s.pair_distribution(2.0, 3.0, 20, 30)
    assert np.array_equal(rad, O.radial32(gx, gy, p.L, 5.0, 50))
    c, sn = O.math32("cos", gth), O.math32("sin", gth)
    assert np.array_equal(pd, O.pair_distribution32(gx, gy, c, sn, 2.0, 3.0, 20, 30))
    # the FP64 restatement of the reference's Pair_Distribution on the same frame
    ref = A.pair_distribution(gx, gy, gth, 2.0, 3.0, 20, 30)
    assert abs(int(pd.sum()) - int(ref.sum())) <= 4 and np.abs(pd.astype(np.int64) - ref).sum() <= 12


def test_radial_distribution_large_system_properties(gpu_lib):
    """N = 1M ABP state: ordered-pair counts are even per unordered pair, the
    disks' repulsion depletes the core, and g(r) -> 1 at larger r."""
    n, L = 1 << 20, 512.0
    p = configs.abp_config(n=n, L=L, seed=1)
    x, y, th = configs.random_state(n, L, seed=1)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(400)
        counts = s.radial_distribution(4.0, 40)
    assert int(counts.sum()) % 2 == 0
    r, g = observables.radial_g(counts, n, L, 4.0)
    assert g[:3].mean() < 0.9 and np.all(np.abs(g[-10:] - 1) < 0.1)


def test_polarization_series_matches_stepwise_readout(gpu_lib):
    p, x, y, th = vicsek_system(n=2048, L=24.0, eta=0.2, seed=3)
    with System(p) as a:
        a.upload(x, y, th)
        pa, pxa, pya = a.polarization_series(30, every=5)
    pb = []
    with System(p) as b:
        b.upload(x, y, th)
        for _ in range(30):
            b.step(5)
            pb.append(b.observables().polarization)
    assert np.array_equal(pa, np.array(pb))
    st = observables.order_parameters(pa, area=4 * p.L * p.L)
    assert st["mean"] == pytest.approx(pa.mean(), rel=1e-12)
    assert 0 <= st["corr_len"] < 15


def test_polarization_series_of_abp_recovers_overflowing_lists(gpu_lib):
    """A series over a run that outgrows its neighbour list: every frame is
    read after the list was grown and the frozen steps re-run."""
    n, L = 4096, 24.0
    p = configs.abp_config(n=n, L=L, seed=2)
    p.list_capacity = 4
    x, y, th = configs.random_state(n, L, seed=2)
    with System(p) as a:
        a.upload(x, y, th)
        pa, _, _ = a.polarization_series(10, every=20)
    q = configs.abp_config(n=n, L=L, seed=2)
    with System(q) as b:
        b.upload(x, y, th)
        pb = []
        for _ in range(10):
            b.step(20)
            pb.append(b.observables().polarization)
    assert np.array_equal(pa, np.array(pb))


def test_batch_binder_matches_series(gpu_lib):
    pts = configs.sweep_points(n_points=3, n_min=300, n_max=1200, seed=5)
    x, y, th = configs.sweep_state(pts, seed=5)
    W, S0, T = 10, 20, 60
    with Batch(pts) as b:
        b.set_windows(W, S0, T)
        b.upload(x, y, th)
        b.step(T)
        st = b.poll()
    for s, p in enumerate(pts):
        sl = slice(b.offsets[s], b.offsets[s + 1])
        state = O.State32(x[sl], y[sl], th[sl])
        P = []
        for t in range(T):
            O.run32(p, state, 1, step0=t)
            P.append(A.frame_polarization(state.th))
        P = np.array(P[S0:])
        m2, m4 = np.mean(P ** 2), np.mean(P ** 4)
        assert st[s].binder == pytest.approx(1 - m4 / (3 * m2 * m2), abs=1e-6)
        assert st[s].binder_reference == pytest.approx(1 - m4 / (3 * m2), abs=1e-6)


def test_system_frames_read_back(gpu_lib, tmp_path):
    """Frames written from the device state (vesicles: membrane beads and
    swimmers) read back through the reference-format reader."""
    from spp_gb300 import binfile
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=8)
    x, y, th = configs.vesicle_state(p)
    path = tmp_path / "traj.bin"
    nm = p.n_rings * p.ring_size
    with System(p) as s, open(path, "wb") as f:
        s.upload(x, y, th)
        states = []
        for _ in range(3):
            s.step(50)
            binfile.write_system_frame(f, s)
            states.append(s.download())
    frames = binfile.read_frames(path)
    assert len(frames) == 3
    for fr, (gx, gy, gth, gix, giy) in zip(frames, states):
        xu = (gx.astype(np.float64) + 2 * p.L * gix).astype(np.float32)
        assert fr.healthy and len(fr.mx) == nm and np.array_equal(fr.mx, xu[:nm])
        assert np.array_equal(fr.x, xu[nm:]) and np.array_equal(fr.theta, gth[nm:])
    assert [fr.t for fr in frames] == pytest.approx([50 * p.dt, 100 * p.dt, 150 * p.dt])


def test_ring_shapes_match_fp64(gpu_lib):
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=8)
    x, y, th = configs.vesicle_state(p)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(200)
        shapes = s.ring_shapes()
        gx, gy, _, gix, giy = s.download()
    xu = gx.astype(np.float64) + 2 * p.L * gix
    yu = gy.astype(np.float64) + 2 * p.L * giy
    M, nr = p.ring_size, p.n_rings
    sw = (p.n - nr * M) // nr
    for r in range(nr):
        mb = A.ring_shape(xu[r * M:(r + 1) * M], yu[r * M:(r + 1) * M])
        q0 = nr * M + r * sw
        swd = A.ring_shape(xu[q0:q0 + sw], yu[q0:q0 + sw])
        for key, v in mb.items():
            assert shapes["mb_" + key][r] == pytest.approx(v, rel=1e-7, abs=1e-7), key
        for key, v in swd.items():
            assert shapes["sw_" + key][r] == pytest.approx(v, rel=1e-7, abs=1e-7), key
        # a ring of 64 beads at rest length 1 stays near-circular: R ~ 10.2, Delta small
        assert 9.0 < shapes["mb_Rg"][r] < 11.5 and shapes["mb_Delta"][r] < 0.05


def test_ring_motion_matches_fp64(gpu_lib):
    """The motion terms of Compute_All_Variables (parallel/beadbox.h:325-434)
    per ring vesicle -- centre-of-mass velocities, angular momenta, rotation
    rates, mean swimmer spin -- between a marked frame and the frame 60 steps
    later, against the FP64 restatement on the same two frames; a second call
    measures from the frame the first one marked."""
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=8)
    x, y, th = configs.vesicle_state(p)
    M, nr = p.ring_size, p.n_rings
    sw = (p.n - nr * M) // nr

    def frame(s):
        gx, gy, gth, gix, giy = s.download()
        return (gx.astype(np.float64) + 2 * p.L * gix, gy.astype(np.float64) + 2 * p.L * giy, gth)

    with System(p) as s:
        s.upload(x, y, th)
        with pytest.raises(SppError):
            s.ring_motion()                 # nothing marked yet
        s.step(100)
        s.ring_motion_mark()
        f0 = frame(s)
        s.step(60)
        m1 = s.ring_motion()
        f1 = frame(s)
        s.step(40)
        m2 = s.ring_motion()
        f2 = frame(s)
    for m, (a, b), steps in ((m1, (f0, f1), 60), (m2, (f1, f2), 40)):
        for r in range(nr):
            q0 = nr * M + r * sw
            mb, swm = slice(r * M, (r + 1) * M), slice(q0, q0 + sw)
            ref = A.ring_motion((b[0][mb], b[1][mb]), (a[0][mb], a[1][mb]), (b[0][swm], b[1][swm]),
                                (a[0][swm], a[1][swm]), b[2][swm], a[2][swm], steps * p.dt)
            for key, v in ref.items():
                assert m[key][r] == pytest.approx(v, rel=1e-9, abs=1e-9), (key, r)
    # swimmers turn at k_perp torque0 and the membranes drift slowly
    assert np.all(np.abs(m1["mb_v_cm_x"]) < 1.0) and np.all(np.isfinite(m1["sw_omega"]))


def test_radial_distribution_in_a_closed_box(gpu_lib):
    """In a closed box pairs are plain differences: particles near opposite
    walls are far apart, not minimum-image neighbours."""
    p = configs.walls_config(n=900, L=20.0)
    x, y, th = configs.walls_state(p)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(200)
        gx, gy, _, _, _ = s.download()
        rad = s.radial_distribution(5.0, 50)
    assert np.array_equal(rad, O.radial32(gx, gy, p.L, 5.0, 50, closed=True))
    assert not np.array_equal(rad, O.radial32(gx, gy, p.L, 5.0, 50))
