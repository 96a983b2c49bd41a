"""Closed boxes with walls on the CPU.

The FP64 restatement of Wall::Interact (shared/wall.h:127-265) is pinned to
the reference's own code where the checkout is present, and everywhere to the
golden fixtures made from it.  The kernels' FP32 wall terms are compared with
the FP64 restatement, a closed box keeps its particles, and the parameters
are validated before any GPU work."""
import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import abi, build, configs

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden import WALL_SEGMENTS, wall_case  # noqa: E402
from test_oracle_pin import load_golden, params_from  # noqa: E402


@pytest.mark.parametrize("name", ["walls_abp", "walls_continuous", "walls_vicsek"])
def test_wall_terms_match_golden(name):
    """RepulsiveParticle force and torque, ContinuousParticle torque, against
    the reference's outputs on 400 particles near four segments."""
    z, meta = load_golden()
    p = params_from(meta[name]["params"])
    pts, ref = z[f"{name}/in"], z[f"{name}/out"]
    got = np.array([O.wall_terms(p, *q) for q in pts])
    assert np.max(np.abs(got - ref) / (1 + np.abs(ref))) < 1e-12
    assert np.count_nonzero(np.any(ref != 0, axis=1)) > 200


@pytest.mark.parametrize("model", [abi.MODEL_ABP, abi.MODEL_CONTINUOUS, abi.MODEL_VICSEK_REF_ANGLE])
def test_wall_terms_match_reference(model):
    if O.ref() is None:
        pytest.skip("reference checkout absent; the golden fixtures pin the walls instead")
    p, _ = wall_case(model)
    rng = np.random.default_rng(5)
    for _ in range(300):
        w = WALL_SEGMENTS[rng.integers(4)]
        u = rng.uniform(-0.3, 1.3)
        x = w[0] + u * (w[2] - w[0]) + rng.uniform(-1.6, 1.6)
        y = w[1] + u * (w[3] - w[1]) + rng.uniform(-1.6, 1.6)
        th = rng.uniform(-np.pi, np.pi)
        a, b = O.wall_terms(p, x, y, th), O.wall_terms(p, x, y, th, fn="ref")
        assert np.all(np.abs(a - b) <= 1e-12 * (1 + np.abs(b)))


@pytest.mark.parametrize("model", [abi.MODEL_ABP, abi.MODEL_CONTINUOUS])
def test_fp32_wall_terms_track_fp64(model):
    """The kernels' FP32 arithmetic (spp_wall_terms, with the FP32 exponential)
    against the FP64 restatement at the same float inputs; the continuous
    torque's perpendicular distance is a difference of nearby numbers, hence
    the looser bound there."""
    p, pts = wall_case(model)
    worst = 0.0
    for x, y, th in pts:
        x, y, th = float(np.float32(x)), float(np.float32(y)), float(np.float32(th))
        a = O.wall_terms(p, x, y, th)
        ref = np.array([a[0], a[1], a[2] if model == abi.MODEL_ABP else a[3]])
        got = O.wall_terms(p, x, y, th, fn="orc32").astype(np.float64)
        worst = max(worst, float(np.max(np.abs(got - ref) / (1 + np.abs(ref)))))
    assert worst < (1e-3 if model == abi.MODEL_ABP else 3e-3)


@pytest.mark.parametrize("integ", [abi.INT_EULER, abi.INT_RK2, abi.INT_RK4])
def test_mirror_tracks_fp64_in_closed_box(integ):
    """ABP in a closed box with two oblique walls: the FP32 mirror stays
    within FP32 rounding of the FP64 restatement, the box keeps every
    particle (no wrap, image counters 0) and the walls did act."""
    p = configs.walls_config(n=900, L=20.0, integrator=integ)
    x, y, th = configs.walls_state(p)
    s32 = O.State32(x, y, th)
    O.run32(p, s32, 300)
    a = O.State64(x.astype(np.float64), y.astype(np.float64), th.astype(np.float64))
    O.run64(p, a, 300)
    assert np.abs(s32.x - a.x).max() < 2e-3 and np.abs(s32.y - a.y).max() < 2e-3
    assert not s32.ix.any() and not s32.iy.any()
    assert np.abs(s32.x).max() < p.L + 0.5 and np.abs(s32.y).max() < p.L + 0.5
    q = p.copy()
    q.A_w = q.g_w = 0.0
    b = O.State64(x.astype(np.float64), y.astype(np.float64), th.astype(np.float64))
    O.run64(q, b, 300)
    assert np.hypot(a.x - b.x, a.y - b.y).max() > 0.05


@pytest.fixture(scope="module")
def lib():
    build.build()
    return abi.lib()


def test_create_rejects_bad_walls_without_touching_gpu(lib):
    p = configs.walls_config(n=64, L=10.0)
    h = C.c_void_p()
    assert lib.spp_create(C.byref(p.replace(boundary=7)), C.byref(h)) == 1
    assert lib.spp_create(C.byref(p.replace(n_walls=5)), C.byref(h)) == 1
    bad = p.copy()
    abi.set_field(bad, "walls", [[1.0, 1.0, 1.0, 1.0]])
    assert lib.spp_create(C.byref(bad), C.byref(h)) == 1
    assert b"nonzero length" in lib.spp_last_error()
    assert lib.spp_create(C.byref(p.replace(sigma_w=0.0)), C.byref(h)) == 1
    v = configs.vicsek_config()
    assert lib.spp_create(C.byref(v.replace(boundary=abi.BOUNDARY_WALLS)), C.byref(h)) == 6
    d = abi.SppParams()
    lib.spp_params_init(C.byref(d), abi.MODEL_CONTINUOUS)
    assert (d.boundary, d.n_walls, d.A_w, d.g_w_cont) == (abi.BOUNDARY_PERIODIC, 0, 0.0, 20.0)


def test_star_trap_segments():
    """Star_Trap_Initialization (shared/set-up.h:259-290) with 2 hands: four
    segments from the tips at r_big to the inner points at r_small."""
    w = np.array(configs.star_trap_walls(2, half_delta=0.3))
    assert w.shape == (4, 4)
    r1 = np.hypot(w[:, 0], w[:, 1])
    r2 = np.hypot(w[:, 2], w[:, 3])
    assert np.allclose(np.sort(np.concatenate([r1, r2])), [6] * 4 + [15] * 4)
    p = configs.walls_config(n=400, L=20.0, extra_walls=configs.star_trap_walls(2))
    x, y, th = configs.walls_state(p)
    s32 = O.State32(x, y, th)
    O.run32(p, s32, 100)
    a = O.State64(x.astype(np.float64), y.astype(np.float64), th.astype(np.float64))
    O.run64(p, a, 100)
    assert np.abs(s32.x - a.x).max() < 1e-3


@pytest.mark.parametrize("model,integ", [(abi.MODEL_ABP, abi.INT_RK2), (abi.MODEL_CONTINUOUS, abi.INT_EULER)])
def test_circular_box_mirror_tracks_fp64(model, integ):
    """The circular box (parallel/box.h:285-294): the kernels' FP32 arithmetic
    (CPU mirror) against the FP64 restatement over 100 steps of particles
    pressed against the circle (the lattice fills it almost to the edge),
    and the circle holds them.  Quantile bounds: a pair the two precisions
    put on different sides of the alignment cutoff parts a few particles by
    more than rounding."""
    p = configs.circle_config(n=1600, L=26.0, model=model, integrator=integ)
    x, y, th = configs.circle_state(p)
    a = O.run64(p, O.State64(x, y, th), 100)
    b = O.run32(p, O.State32(x, y, th), 100)
    r64 = np.hypot(a.x, a.y)
    assert r64.max() < p.L and (r64 > p.L - 1).sum() > 0   # the circle torque acted
    err = np.maximum(np.abs(b.x - a.x), np.abs(b.y - a.y))
    assert np.quantile(err, 0.99) < 1e-4 and err.max() < 0.01
    assert np.all(b.ix == 0) and np.all(b.iy == 0)


def test_circle_torque_formula():
    """The FP32 circle torque against the formula of parallel/box.h:292,
    40 g (v_y x - v_x y) / (2 pi r (L - r)), evaluated in FP64."""
    p = configs.circle_config(n=8, L=10.0)
    rng = np.random.default_rng(3)
    for _ in range(200):
        r = rng.uniform(8.5, 9.99)
        phi, th = rng.uniform(-np.pi, np.pi, 2)
        x, y = np.float32(r * np.cos(phi)), np.float32(r * np.sin(phi))
        th = np.float32(th)
        got = O.circle_torque32(p, x, y, th)
        xd, yd = float(x), float(y)
        rd = np.hypot(xd, yd)
        want = 40 * p.g * (np.sin(th) * xd - np.cos(th) * yd) / (2 * np.pi * rd * (p.L - rd))
        if not rd > p.L - 1:
            want = 0.0
        assert abs(got - want) <= 1e-4 * (1 + abs(want)), (got, want)
    assert O.circle_torque32(p, np.float32(3.0), np.float32(4.0), np.float32(0.3)) == 0.0


def test_vicsek_wall_alignment_fp32_vs_fp64():
    """VicsekParticle's wall term (shared/wall.h:163-190): the kernels' FP32
    count and folded angle against the FP64 restatement at the same float
    inputs.  The count may differ only where the distance or the foot lies
    within rounding of its bound; the angle within FP32 rounding except next
    to a fold (dtheta = +-pi/2), where the two may fold differently."""
    p, pts = wall_case(abi.MODEL_VICSEK_REF_ANGLE)
    bad_cnt = 0
    hits = 0
    for x, y, th in pts:
        x, y, th = float(np.float32(x)), float(np.float32(y)), float(np.float32(th))
        a = O.wall_terms(p, x, y, th)
        b = O.wall_terms(p, x, y, th, fn="orc32")
        if a[0] != b[0]:
            bad_cnt += 1
            continue
        hits += a[0] > 0
        if a[0] > 0:
            d = abs(a[1] - b[1])
            assert d < 1e-5 or abs(d - np.pi) < 1e-5 * a[0], (x, y, th, a, b)
    assert bad_cnt <= 2 and hits > 100


def test_vicsek_walls_mirror_tracks_fp64():
    """VicsekParticle (angle average) in a closed box with two oblique
    segments across the flock: the FP32 mirror against the FP64 restatement
    over 10 steps (the angle average is well conditioned; walls add
    neighbours and angles)."""
    p = configs.walls_config(n=2000, L=60.0, model=abi.MODEL_VICSEK_REF_ANGLE, seed=4)
    x, y, th = configs.vicsek_walls_state(p)
    a = O.run64(p, O.State64(x, y, th), 10)
    b = O.run32(p, O.State32(x, y, th), 10)
    e = np.abs((b.th.astype(np.float64) - a.th + np.pi) % (2 * np.pi) - np.pi)
    assert np.quantile(e, 0.99) < 1e-5 and np.max(np.abs(b.x - a.x)) < 1e-3
