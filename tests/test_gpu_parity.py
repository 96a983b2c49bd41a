"""GPU parity through the C ABI.

Gate 1 (bit-exact): the kernels against the CPU mirror of their arithmetic
(oracle/spp_mirror32.c) -- same Philox draws, same FP32 formulas,
order-independent fixed-point sums -- so any difference is a fault in the
device machinery (binning, Morton reordering, Verlet lists and their
displacement trigger, graphs).
Gate 2 (tolerance): the kernels against the FP64 restatement of the
reference (oracle/spp_oracle64.c, itself pinned to the reference's code).
Tolerance from the spec: positions and headings within 1e-5 relative over
100 steps, except where FP32 and FP64 disagree on which pairs lie inside a
hard cutoff (alignment radius); those particles are counted and bounded.
"""
import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import System, abi, configs

pytestmark = pytest.mark.gpu


def run_gpu(p, x, y, th, steps, step0=0):
    with System(p) as s:
        s.upload(x, y, th, step0=step0)
        s.step(steps)
        out = s.download()
        obs = s.observables()
    return out, obs


def assert_bitexact(gpu, mirror):
    gx, gy, gth, gix, giy = gpu
    for name, a, b in (("x", gx, mirror.x), ("y", gy, mirror.y), ("theta", gth, mirror.th),
                       ("img_x", gix, mirror.ix), ("img_y", giy, mirror.iy)):
        bad = np.flatnonzero(a != b)
        assert bad.size == 0, f"{name}: {bad.size} particles differ, first {bad[:5]}"


def lattice(n_side, L, jitter_seed=None):
    g = (np.arange(n_side) * (2 * L / n_side) - L + 0.25).astype(np.float32)
    X, Y = np.meshgrid(g, g)
    return X.ravel().astype(np.float32), Y.ravel().astype(np.float32)


ABP_CASES = {
    "abp_harmonic_mean_rk2": dict(integrator=abi.INT_RK2, steps=100),
    "abp_harmonic_mean_rk4": dict(integrator=abi.INT_RK4, steps=60),
    "abp_harmonic_mean_euler": dict(integrator=abi.INT_EULER, steps=60),
}


@pytest.mark.parametrize("case", sorted(ABP_CASES))
def test_abp_bitexact_vs_mirror(gpu_lib, case):
    c = ABP_CASES[case]
    p = configs.abp_config(n=4096, L=32.0, seed=1, integrator=c["integrator"])
    x, y, th = configs.random_state(p.n, p.L, seed=1)
    gpu, obs = run_gpu(p, x, y, th, c["steps"])
    ref = O.run32(p, O.State32(x, y, th), c["steps"])
    assert_bitexact(gpu, ref)
    assert obs.step == c["steps"]
    assert obs.n_rebuilds >= 2  # the displacement trigger fired during the run


@pytest.mark.parametrize("integ", [abi.INT_RK2, abi.INT_RK4, abi.INT_EULER])
def test_repulsive_reference_mode_bitexact(gpu_lib, integ):
    """RepulsiveParticle as shipped: R12 force, g sin / (pi R_a^2), f = v."""
    p = configs.reference_defaults(abi.MODEL_ABP)
    p.n, p.L, p.Dr, p.dt, p.seed, p.integrator, p.skin = 4096, 32.0, 0.1, 0.005, 5, integ, 0.3
    x, y = lattice(64, p.L)
    _, _, th = configs.random_state(p.n, p.L, seed=7)
    gpu, _ = run_gpu(p, x, y, th, 60)
    ref = O.run32(p, O.State32(x, y, th), 60)
    assert_bitexact(gpu, ref)


@pytest.mark.parametrize("model", [abi.MODEL_VICSEK, abi.MODEL_VICSEK_REF_ANGLE,
                                   abi.MODEL_VICSEK_REF_VECTOR])
def test_vicsek_bitexact_vs_mirror(gpu_lib, model):
    p = configs.vicsek_config(model=model)
    x, y, th = configs.random_state(p.n, p.L, seed=0)
    gpu, obs = run_gpu(p, x, y, th, 100)
    ref = O.run32(p, O.State32(x, y, th), 100)
    assert_bitexact(gpu, ref)
    P, _, _ = O.polarization(ref.th)
    assert abs(obs.polarization - P) < 1e-6


@pytest.mark.parametrize("model", [abi.MODEL_VICSEK, abi.MODEL_VICSEK_REF_ANGLE,
                                   abi.MODEL_VICSEK_REF_VECTOR])
def test_vicsek_single_block_path_matches_multi_kernel_path(gpu_lib, model, monkeypatch):
    """Small systems run whole steps in one block (k_vicsek_small); the
    multi-kernel step (SPP_VICSEK_SMALL=0) and the mirror give the same
    bits, including the box-crossing counters, for several calls of
    different lengths and a system at the size limit."""
    for n, L in ((4096, 32.0), (8192, 40.0)):
        p = configs.vicsek_config(model=model)
        p.n, p.L = n, L
        x, y, th = configs.random_state(p.n, p.L, seed=5)
        outs = []
        for small in ("1", "0"):
            monkeypatch.setenv("SPP_VICSEK_SMALL", small)
            with System(p) as s:
                s.upload(x, y, th, step0=17)
                s.step(1)
                s.step(40)
                s.step(159)
                outs.append(s.download())
        for a, b in zip(*outs):
            assert np.array_equal(a, b)
        ref = O.run32(p, O.State32(x, y, th), 200, step0=17)
        assert_bitexact(outs[0], ref)
        assert np.abs(outs[0][3]).max() > 0  # particles crossed the boundary


@pytest.mark.parametrize("integ", [abi.INT_EULER, abi.INT_RK4])
def test_continuous_bitexact_vs_mirror(gpu_lib, integ):
    p = configs.reference_defaults(abi.MODEL_CONTINUOUS)
    p.n, p.L, p.dt, p.v0, p.seed, p.skin, p.integrator = 4096, 32.0, 0.01, 0.5, 3, 0.3, integ
    if integ == abi.INT_RK4:  # continuous-time Vicsek of the Lyapunov workload
        p.alpha, p.g, p.Dr = 0.0, 1.0, 0.0
    else:
        p.Dr = 0.05
    x, y, th = configs.random_state(p.n, p.L, seed=2)
    gpu, _ = run_gpu(p, x, y, th, 50)
    ref = O.run32(p, O.State32(x, y, th), 50)
    assert_bitexact(gpu, ref)


def reference_lattice_abp(integrator):
    """RepulsiveParticle as shipped (R12 force, g sin / (pi R_a^2)) on a
    lattice start: the R12 law does not admit the overlaps of a uniform
    random start."""
    p = configs.reference_defaults(abi.MODEL_ABP)
    p.n, p.L, p.Dr, p.dt, p.seed, p.integrator, p.skin = 4096, 32.0, 0.1, 0.005, 5, integrator, 0.3
    x, y = lattice(64, p.L)
    _, _, th = configs.random_state(p.n, p.L, seed=7)
    return p, x, y, th


def continuous_alpha0(integrator):
    """ContinuousParticle with alpha = 0, g = 1 (the Lyapunov workload's
    model) and rotational noise D_r = 0.05."""
    p = configs.lyapunov_config(n=4096)
    p.integrator, p.Dr = integrator, 0.05
    x, y, th = configs.random_state(p.n, p.L, seed=2)
    return p, x, y, th


def continuous_reference(integrator):
    """ContinuousParticle with the reference's defaults (g = 4, alpha = 0.5,
    dt = 2^-10, shared/particle.h:373-378) and D_r = 0.05."""
    p = configs.reference_defaults(abi.MODEL_CONTINUOUS)
    p.n, p.L, p.seed, p.skin, p.integrator, p.Dr = 4096, 32.0, 3, 0.3, integrator, 0.05
    x, y, th = configs.random_state(p.n, p.L, seed=2)
    return p, x, y, th


def harmonic_abp(integrator):
    """The configured repulsive ABP/Vicsek physics (harmonic k(1 - r/2a),
    (g/n_i) sum sin alignment) at N = 4096."""
    p = configs.abp_config(n=4096, L=32.0, seed=1, integrator=integrator)
    x, y, th = configs.random_state(p.n, p.L, seed=1)
    return p, x, y, th


TWO_PI = 2.0 * np.pi
# case: (state maker, integrator, alignment hops exempted, close-approach radius, heading tolerance)
FP64_CASES = {
    "abp_harmonic_rk2": (harmonic_abp, abi.INT_RK2, 1, 0.0, 1e-5),
    "abp_harmonic_rk4": (harmonic_abp, abi.INT_RK4, 1, 0.0, 1e-5),
    "abp_r12_reference_euler": (reference_lattice_abp, abi.INT_EULER, 1, 0.0, 1e-5),
    "abp_r12_reference_rk2": (reference_lattice_abp, abi.INT_RK2, 1, 0.0, 1e-5),
    "abp_r12_reference_rk4": (reference_lattice_abp, abi.INT_RK4, 1, 0.0, 1e-5),
    "continuous_alpha0_euler": (continuous_alpha0, abi.INT_EULER, 2, 0.0, 1e-5),
    "continuous_alpha0_rk2": (continuous_alpha0, abi.INT_RK2, 2, 0.0, 1e-5),
    "continuous_alpha0_rk4": (continuous_alpha0, abi.INT_RK4, 2, 0.0, 1e-5),
    "continuous_reference_euler": (continuous_reference, abi.INT_EULER, 2, 0.02, 1e-5 * TWO_PI),
    "continuous_reference_rk2": (continuous_reference, abi.INT_RK2, 2, 0.02, 1e-5 * TWO_PI),
    "continuous_reference_rk4": (continuous_reference, abi.INT_RK4, 2, 0.02, 1e-5 * TWO_PI),
}


@pytest.mark.parametrize("case", sorted(FP64_CASES))
def test_vs_fp64_100_steps(gpu_lib, case):
    """The kernels against the FP64 restatement of the reference (itself
    pinned bit for bit, or to 1e-11, to the reference's own particle.h) over
    100 steps at N = 4096: every particle within 1e-5 of the box side in
    position and within the case's tolerance in heading, except those a hard
    cutoff legitimately separates.

    Where FP32 and FP64 put a pair on different sides of the alignment
    radius (found by recording, in both precisions, every evaluation within
    1e-3 of the cutoff: oracle.cutoff_divergence), the two particles' torques
    jump by ~ dt g / n_i and their headings part by far more than rounding;
    their neighbours feel that through their own alignment sums.  Exempt
    are the members of such pairs and the particles within `hops` alignment
    radii of them afterwards (hops = 2 for the continuous model, whose
    torque g sum sin / pi is not normalised by the neighbour count).  The
    continuous model's alpha torque alpha (dr x v) / (pi d) takes its
    direction from dr / d; with no repulsion, pairs pass through each other,
    and FP32's position resolution near |x| ~ L (2e-6) then moves headings
    by ~ 1e-5 over 100 steps at distances ~ 0.1: pairs closer than 0.02 are
    exempt, and headings are held to 1e-5 of a full turn there.  The GPU is
    first shown bit-identical to the FP32 mirror whose cutoff decisions are
    recorded, so those decisions are the kernels' own."""
    make, integ, hops, close, th_tol = FP64_CASES[case]
    p, x, y, th = make(integ)
    steps = 100
    gpu, _ = run_gpu(p, x, y, th, steps)
    s64, s32, mism, level = O.cutoff_divergence(p, x, y, th, steps, hops=hops, close=close)
    assert_bitexact(gpu, s32)
    gx, gy, gth, gix, giy = gpu
    xu = gx.astype(np.float64) + 2 * p.L * gix
    yu = gy.astype(np.float64) + 2 * p.L * giy
    rel_pos = np.maximum(np.abs(xu - s64.xu), np.abs(yu - s64.yu)) / (2 * p.L)
    dth = np.abs((gth.astype(np.float64) - s64.th + np.pi) % TWO_PI - np.pi)
    ok = level > hops
    print(f"{case}: {mism.size} FP32/FP64 cutoff mismatches, {np.sum(~ok)} of {p.n} particles exempt; "
          f"others: max |dr|/2L {rel_pos[ok].max():.3g}, max |dtheta| {dth[ok].max():.3g}, "
          f"median |dtheta| {np.median(dth[ok]):.3g}; all: max |dr|/2L {rel_pos.max():.3g}, "
          f"max |dtheta| {dth.max():.3g}")
    assert rel_pos[ok].max() <= 1e-5
    assert dth[ok].max() <= th_tol
    assert np.mean(~ok) < 0.1


def werr(a, b, period):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return np.abs((d + period / 2) % period - period / 2)


@pytest.mark.parametrize("model,steps", [(abi.MODEL_VICSEK, 10), (abi.MODEL_VICSEK_REF_ANGLE, 10),
                                         (abi.MODEL_VICSEK_REF_VECTOR, 5)])
def test_vicsek_vs_fp64_short_horizon(gpu_lib, model, steps):
    """The discrete Vicsek models (config-1 rule, VicsekParticle's angle
    average, VicsekParticle2's vector sum with push, shared/particle.h:
    145-250) against the FP64 restatement.  At dt = 1 they are chaotic: a
    heading sum that nearly cancels (the vector rules) turns rounding
    differences into large heading differences, and a pair crossing the
    cutoff differently moves a particle by a whole step.  So the horizon is
    short and the bounds are quantiles: the angle average (well conditioned)
    keeps every particle within 1e-5 over 10 steps."""
    p = configs.vicsek_config(model=model)
    x, y, th = configs.random_state(p.n, p.L, seed=0)
    (gx, gy, gth, gix, giy), _ = run_gpu(p, x, y, th, steps)
    a = O.run64(p, O.State64(x, y, th), steps)
    e = werr(gth, a.th, TWO_PI)
    xu = gx.astype(np.float64) + 2 * p.L * gix
    yu = gy.astype(np.float64) + 2 * p.L * giy
    ep = np.maximum(np.abs(xu - a.xu), np.abs(yu - a.yu)) / (2 * p.L)
    print(f"model {model}, {steps} steps: |dtheta| median {np.median(e):.3g}, q90 {np.quantile(e, 0.9):.3g}, "
          f"q99 {np.quantile(e, 0.99):.3g}, max {e.max():.3g}, > 1e-5 at {np.mean(e > 1e-5):.2%}; "
          f"|dr|/2L q99 {np.quantile(ep, 0.99):.3g}, max {ep.max():.3g}")
    if model == abi.MODEL_VICSEK_REF_ANGLE:
        assert e.max() <= 1e-5 and ep.max() <= 1e-5
    elif model == abi.MODEL_VICSEK:
        assert np.median(e) < 1e-6 and np.quantile(e, 0.99) < 1e-5 and e.max() < 1e-3
        assert np.mean(e > 1e-5) < 0.02 and np.quantile(ep, 0.99) < 1e-5
    else:
        assert np.median(e) < 1e-6 and np.quantile(e, 0.9) < 1e-5 and e.max() < 1e-2
        assert np.mean(e > 1e-5) < 0.05 and np.quantile(ep, 0.99) < 1e-5


def test_pairs_bitexact_vs_mirror(gpu_lib):
    p = configs.abp_config(n=4096, L=32.0, seed=1)
    x, y, th = configs.random_state(p.n, p.L, seed=3)
    with System(p) as s:
        s.upload(x, y, th)
        for r in (1.0, 1.3):
            g = s.pairs(r)
            m = O.pairs32(p, x, y, r)
            assert np.array_equal(g, m), r
            k64 = O.pairs64(x.astype(np.float64), y.astype(np.float64), p.L, r)
            assert np.setxor1d(g, k64).size <= 2
        s.step(50)
        gx, gy, _, _, _ = s.download()
        assert np.array_equal(s.pairs(1.0), O.pairs32(p, gx, gy, 1.0))


def test_cells_bitexact_vs_mirror(gpu_lib):
    p = configs.abp_config(n=4096, L=32.0, seed=1)
    x, y, th = configs.random_state(p.n, p.L, seed=3)
    with System(p) as s:
        s.upload(x, y, th)
        for D in (3, 49, 64):
            for rule in (abi.BIN_GEOMETRIC, abi.BIN_REFERENCE):
                gx, gy = s.cells(D, rule)
                mx, my = O.cells32(p, x, y, D, rule)
                assert np.array_equal(gx, mx) and np.array_equal(gy, my), (D, rule)


def test_full_size_abp_bitexact_vs_mirror(gpu_lib):
    """The headline workload's size (N = 1,048,576, L = 512): 10 RK2 steps."""
    p = configs.abp_config()
    x, y, th = configs.random_state(p.n, p.L, seed=1)
    gpu, obs = run_gpu(p, x, y, th, 10)
    ref = O.run32(p, O.State32(x, y, th), 10)
    assert_bitexact(gpu, ref)
    assert obs.cells_per_side == int(np.floor(1024 / (1.3 * 1.001)))


def test_full_size_abp_properties(gpu_lib):
    """Size-independent properties over 400 steps of the full workload:
    positions stay wrapped, headings finite, deterministic replay, and the
    unwrapped displacement is bounded by v0 t plus the force contribution."""
    p = configs.abp_config()
    x, y, th = configs.random_state(p.n, p.L, seed=1)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(400)
        a = s.download()
        o = s.observables()
    with System(p) as s:
        s.upload(x, y, th)
        s.step(200)
        s.step(200)
        b = s.download()
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    gx, gy, gth, gix, giy = a
    assert np.all(np.isfinite(gth))
    assert np.all((gx >= -p.L) & (gx < p.L) & (gy >= -p.L) & (gy < p.L))
    xu = gx.astype(np.float64) + 2 * p.L * gix - x
    yu = gy.astype(np.float64) + 2 * p.L * giy - y
    disp = np.hypot(xu, yu)
    assert disp.max() < 400 * p.dt * 8.0
    assert 0.0 <= o.polarization <= 1.0
    assert o.n_rebuilds > 3


@pytest.mark.parametrize("lanes", [1, 4])
@pytest.mark.parametrize("integ", [abi.INT_RK2, abi.INT_RK4])
def test_vesicles_bitexact_vs_mirror(gpu_lib, integ, lanes):
    """Ring membranes (bonds + bending) with swimmers, bit-exact against the
    mirror, with one or four threads per body in the neighbour sums."""
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=16, L=48.0,
                               integrator=integ)
    p.gather_lanes = lanes
    x, y, th = configs.vesicle_state(p)
    gpu, obs = run_gpu(p, x, y, th, 150)
    ref = O.run32(p, O.State32(x, y, th), 150)
    assert_bitexact(gpu, ref)
    assert obs.late_rebuilds == 0


def test_vesicles_full_size_bitexact_vs_mirror(gpu_lib):
    """The full vesicle workload: 1024 rings x 128 beads + 32,768 swimmers, RK4."""
    p = configs.vesicle_config()
    x, y, th = configs.vesicle_state(p)
    gpu, obs = run_gpu(p, x, y, th, 4)
    ref = O.run32(p, O.State32(x, y, th), 4)
    assert_bitexact(gpu, ref)


def test_vesicles_vs_fp64(gpu_lib):
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=16, L=48.0)
    x, y, th = configs.vesicle_state(p)
    (gx, gy, gth, gix, giy), _ = run_gpu(p, x, y, th, 100)
    a = O.run64(p, O.State64(x, y, th), 100)
    xu = gx.astype(np.float64) + 2 * p.L * gix
    yu = gy.astype(np.float64) + 2 * p.L * giy
    nb = p.n_rings * p.ring_size
    assert np.max(np.abs(xu - a.xu)) / (2 * p.L) < 1e-5
    assert np.max(np.abs(yu - a.yu)) / (2 * p.L) < 1e-5
    dth = np.abs((gth[nb:].astype(np.float64) - a.th[nb:] + np.pi) % (2 * np.pi) - np.pi)
    assert np.max(dth) < 1e-5


@pytest.mark.parametrize("integ", [abi.INT_EULER, abi.INT_RK2, abi.INT_RK4])
def test_run_and_tumble_bitexact_vs_mirror(gpu_lib, integ):
    """RTPChain swimmers (run and tumble) inside ring membranes: the tumble
    states live by particle id on the device and advance once per step."""
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=16, L=48.0,
                               integrator=integ, seed=9)
    x, y, th = configs.vesicle_state(p)
    p.rot_noise = abi.NOISE_TUMBLE
    p.tumble_rate, p.tumble_time, p.tumble_torque = 20.0, 0.03, 3.0
    if integ == abi.INT_EULER:
        p.dt = 0.0005  # the stiff bonds and bending need a smaller first-order step
    gpu, _ = run_gpu(p, x, y, th, 200)
    ref = O.run32(p, O.State32(x, y, th), 200)
    assert_bitexact(gpu, ref)
    nb = p.n_rings * p.ring_size
    assert np.abs(gpu[2][nb:] - th[nb:]).max() > 0.1


def test_run_and_tumble_fraction_of_time_tumbling(gpu_lib):
    """Many free swimmers: the stationary share of tumbling swimmers is
    rate * T / (1 + rate * T) with T the tumble length (the geometric
    waiting time of the start draws)."""
    p = configs.vesicle_config(n_rings=0, ring_size=3, swimmers_per_ring=0, L=200.0, seed=4)
    p.n = 40000
    p.force_law = abi.FORCE_NONE  # random placement: no overlapping pairs to resolve
    x, y, th = configs.random_state(p.n, p.L, seed=4)
    p.rot_noise = abi.NOISE_TUMBLE
    p.tumble_rate, p.tumble_time, p.tumble_torque, p.dt = 5.0, 0.1, 2.0, 0.002
    K = O.tumble_steps(p)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(2000)
        t1 = s.download()[2].astype(np.float64)
        s.step(1)
        t2 = s.download()[2].astype(np.float64)
    dth = np.abs(((t2 - t1) + np.pi) % (2 * np.pi) - np.pi)
    turning = dth > 0.5 * p.k_perp * p.dt * p.tumble_torque
    rate_dt = p.tumble_rate * p.dt
    # per step: a running swimmer starts with probability rate*dt; a tumble
    # turns for K steps (start step included) and resets on the next
    expect = K / (K + 1 + 1 / rate_dt - 1)
    assert abs(turning.mean() - expect) < 0.02, (turning.mean(), expect)


@pytest.mark.parametrize("integ", [abi.INT_EULER, abi.INT_RK2, abi.INT_RK4])
def test_chains_bitexact_vs_mirror(gpu_lib, integ):
    """Free chiral trimers (ActiveBrownianChain with nb = 3): the bead-pair
    R12 forces and lever-arm torques summed in list order, the anisotropic
    mobility of Set_nb, and Move()'s projection on the turned heading."""
    p = configs.chain_config(n=4096, chain_beads=3, integrator=integ, seed=6, spacing=1.7)
    p.torque0 = 0.3
    x, y, th = configs.chain_state(p)
    gpu, obs = run_gpu(p, x, y, th, 300)
    ref = O.run32(p, O.State32(x, y, th), 300)
    assert_bitexact(gpu, ref)
    assert obs.n_rebuilds >= 1


@pytest.mark.parametrize("tumble", [False, True])
def test_dimers_in_vesicles_bitexact_vs_mirror(gpu_lib, tumble):
    """Dimer swimmers (nb = 2, the default chain length of the reference's
    membrane driver) inside ring membranes: membrane-membrane pairs by the
    membrane law, every pair with a dimer by the chain law; optionally run
    and tumble with the dimers' own k_perpendicular."""
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=16, L=48.0, seed=9)
    x, y, th = configs.vesicle_state(p)
    p.chain_beads, p.bead_separation, p.sigma_chain, p.r_chain = 2, 0.5, 0.5, 0.55
    if tumble:
        p.rot_noise = abi.NOISE_TUMBLE
        p.tumble_rate, p.tumble_time, p.tumble_torque = 20.0, 0.03, 3.0
    gpu, _ = run_gpu(p, x, y, th, 200)
    ref = O.run32(p, O.State32(x, y, th), 200)
    assert_bitexact(gpu, ref)


def clustered_state(n, L, clusters, seed):
    """Uniform background plus tight clusters (sizes, radius 0.35): lists of
    every length class, from a few entries to beyond 512."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-L, L, n)
    y = rng.uniform(-L, L, n)
    th = rng.uniform(-np.pi, np.pi, n)
    start = 0
    centres = [(-0.5 * L, -0.5 * L), (0.5 * L, -0.5 * L), (-0.5 * L, 0.5 * L), (0.5 * L, 0.5 * L),
               (0.0, 0.0), (0.0, 0.5 * L)]
    for size, (cx, cy) in zip(clusters, centres):
        r = 0.35 * np.sqrt(rng.uniform(0, 1, size))
        a = rng.uniform(0, 2 * np.pi, size)
        x[start:start + size] = cx + r * np.cos(a)
        y[start:start + size] = cy + r * np.sin(a)
        start += size
    return x.astype(np.float32), y.astype(np.float32), th.astype(np.float32)


@pytest.mark.parametrize("n", [4096, 20000])
def test_long_lists_bitexact_vs_mirror(gpu_lib, n):
    """Clusters of 700, 300, 150, 100, 60 and 28 particles in a sparse background:
    lists longer than the 12 shared-memory keys are finished in place up to
    16 entries, then by the warp bitonic sort (32 to 512 keys) and beyond 512
    by the one-lane fallback; the list overflows and regrows on the way.
    4096 particles use four lanes per particle, 20,000 one."""
    p = configs.reference_defaults(abi.MODEL_CONTINUOUS)
    p.n, p.L, p.dt, p.v0, p.seed, p.skin, p.integrator = n, 40.0, 0.01, 0.2, 3, 0.3, abi.INT_RK2
    p.Dr = 0.05
    x, y, th = clustered_state(p.n, p.L, (700, 300, 150, 100, 60, 28), seed=8)
    gpu, obs = run_gpu(p, x, y, th, 30)
    ref = O.run32(p, O.State32(x, y, th), 30)
    assert_bitexact(gpu, ref)
    assert obs.max_neighbors > 600


@pytest.mark.parametrize("model,integ", [(abi.MODEL_ABP, abi.INT_EULER), (abi.MODEL_ABP, abi.INT_RK2),
                                         (abi.MODEL_ABP, abi.INT_RK4), (abi.MODEL_CONTINUOUS, abi.INT_EULER),
                                         (abi.MODEL_CONTINUOUS, abi.INT_RK2)])
@pytest.mark.parametrize("n", [4096, 20000])
def test_walls_bitexact_vs_mirror(gpu_lib, model, integ, n):
    """Closed box with two oblique walls (Wall::Interact of
    RepulsiveParticle / ContinuousParticle): no wrap, no minimum image, the
    wall terms after the pair sums; four lanes per particle at 4096, one at
    20,000."""
    L = 40.0 if n == 4096 else 80.0
    p = configs.walls_config(n=n, L=L, model=model, integrator=integ)
    x, y, th = configs.walls_state(p)
    steps = 150
    gpu, _ = run_gpu(p, x, y, th, steps)
    ref = O.run32(p, O.State32(x, y, th), steps)
    assert_bitexact(gpu, ref)
    assert not gpu[3].any() and not gpu[4].any()


@pytest.mark.parametrize("model,integ", [(abi.MODEL_ABP, abi.INT_RK2), (abi.MODEL_ABP, abi.INT_RK4),
                                         (abi.MODEL_CONTINUOUS, abi.INT_EULER),
                                         (abi.MODEL_CONTINUOUS, abi.INT_RK2)])
@pytest.mark.parametrize("n", [4096, 20000])
def test_circular_box_bitexact_vs_mirror(gpu_lib, model, integ, n):
    """Circular box (parallel/box.h:285-294): no wrap, no minimum image, the
    circle's torque on particles beyond r = L - 1; four lanes per particle
    at 4096, one at 20,000.  After 600 more steps the circle still holds
    the particles: it turns them back but does not push, so the repulsion
    of the crowd behind can press a few across it, as in the reference."""
    L = 40.0 if n == 4096 else 86.0
    p = configs.circle_config(n=n, L=L, model=model, integrator=integ)
    x, y, th = configs.circle_state(p)
    gpu, _ = run_gpu(p, x, y, th, 150)
    ref = O.run32(p, O.State32(x, y, th), 150)
    assert_bitexact(gpu, ref)
    assert not gpu[3].any() and not gpu[4].any()
    with System(p) as s:
        s.upload(*gpu[:3])
        s.step(600)
        gx, gy, _, _, _ = s.download()
    r = np.hypot(gx.astype(np.float64), gy.astype(np.float64))
    assert np.mean(r < p.L) > 0.99 and r.max() < p.L + 2.0


@pytest.mark.parametrize("model", [abi.MODEL_VICSEK_REF_ANGLE, abi.MODEL_VICSEK_REF_VECTOR])
@pytest.mark.parametrize("n,L", [(2000, 60.0), (30000, 240.0)])
def test_vicsek_walls_bitexact_vs_mirror(gpu_lib, model, n, L):
    """The discrete Vicsek models in a closed box with two oblique segments:
    VicsekParticle counts a wall within distance 1 as a neighbour and adds
    its folded relative heading (Wall::Interact(VicsekParticle*),
    shared/wall.h:163-190); VicsekParticle2 has no wall overload (the empty
    Wall::Interact(BasicDynamicParticle*), :159-161), so only the closed box
    acts on it.  2000 particles run in the one-cluster kernel, 30,000 through
    the multi-kernel step."""
    p = configs.walls_config(n=n, L=L, model=model, seed=4,
                             extra_walls=((-10.0, -4.0, 8.0, 12.0), (6.0, -14.0, -12.0, 2.0)))
    x, y, th = configs.vicsek_walls_state(p, half=30.0 if n == 2000 else 110.0)
    gpu, _ = run_gpu(p, x, y, th, 30)
    ref = O.run32(p, O.State32(x, y, th), 30)
    assert_bitexact(gpu, ref)
    assert not gpu[3].any() and not gpu[4].any()


def test_star_trap_bitexact_vs_mirror(gpu_lib):
    """ABP in a closed box holding a two-hand star trap (four segments)."""
    p = configs.walls_config(n=2500, L=30.0, extra_walls=configs.star_trap_walls(2))
    x, y, th = configs.walls_state(p)
    gpu, _ = run_gpu(p, x, y, th, 200)
    ref = O.run32(p, O.State32(x, y, th), 200)
    assert_bitexact(gpu, ref)
