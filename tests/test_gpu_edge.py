"""Edge cases through the C ABI on the GPU: tiny and ragged systems,
boundary coordinates, neighbour-list overflow and its recovery, graph vs
direct launches, invalid inputs, fixed-point overflow."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import SppError, System, abi, configs

pytestmark = pytest.mark.gpu


def gpu_run(p, x, y, th, steps):
    with System(p) as s:
        s.upload(x, y, th)
        s.step(steps)
        return s.download(), s.observables()


def same(gpu, ref):
    gx, gy, gth, gix, giy = gpu
    return (np.array_equal(gx, ref.x) and np.array_equal(gy, ref.y) and np.array_equal(gth, ref.th)
            and np.array_equal(gix, ref.ix) and np.array_equal(giy, ref.iy))


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 257, 1000])
def test_ragged_sizes_bitexact(gpu_lib, n):
    p = configs.abp_config(n=n, L=4.0, seed=2)
    x, y, th = configs.random_state(n, p.L, seed=n)
    gpu, _ = gpu_run(p, x, y, th, 40)
    assert same(gpu, O.run32(p, O.State32(x, y, th), 40))


def test_boundary_coordinates(gpu_lib):
    L = np.float32(8.0)
    edge = np.nextafter(L, np.float32(0))
    x = np.array([-L, edge, 0.0, -L, edge, 0.5], np.float32)
    y = np.array([-L, -L, edge, edge, 0.0, 0.5], np.float32)
    th = np.array([3.1, -3.1, 1.5, -1.5, 0.0, 2.0], np.float32)
    p = configs.abp_config(n=6, L=8.0, seed=3)
    gpu, _ = gpu_run(p, x, y, th, 200)
    assert same(gpu, O.run32(p, O.State32(x, y, th), 200))
    v = configs.vicsek_config(n=6, L=8.0)
    gpu, _ = gpu_run(v, x, y, th, 50)
    assert same(gpu, O.run32(v, O.State32(x, y, th), 50))


def test_dense_cluster_list_overflow_recovers(gpu_lib):
    """512 aligning particles (no repulsion) in a 2x2 patch overflow a 4-slot
    list: the device freezes, the host grows the list and finishes the
    steps; the result stays bit-exact."""
    n = 512
    p = configs.abp_config(n=n, L=16.0, seed=4)
    p.force_law = abi.FORCE_NONE
    p.list_capacity = 4
    x, y, th = configs.random_state(n, 1.0, seed=4)
    gpu, obs = gpu_run(p, x, y, th, 30)
    assert obs.list_capacity > 4
    assert obs.max_neighbors > 400
    assert obs.step == 30 and obs.late_rebuilds == 0
    assert same(gpu, O.run32(p, O.State32(x, y, th), 30))


def test_exploding_cluster_reports_late_rebuilds(gpu_lib):
    """512 overlapping harmonic disks fly apart at ~15 length units per step,
    far beyond the skin: the device counts the rebuilds that came too late
    instead of failing silently."""
    n = 512
    p = configs.abp_config(n=n, L=16.0, seed=4)
    x, y, th = configs.random_state(n, 1.0, seed=4)
    _, obs = gpu_run(p, x, y, th, 5)
    assert obs.late_rebuilds > 0


def test_graphs_and_direct_launches_agree(gpu_lib, monkeypatch):
    p = configs.abp_config(n=4096, L=32.0, seed=6)
    x, y, th = configs.random_state(p.n, p.L, seed=6)
    a, _ = gpu_run(p, x, y, th, 70)
    monkeypatch.setenv("SPP_NO_GRAPHS", "1")
    b, _ = gpu_run(p, x, y, th, 70)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_step0_offsets_the_noise_stream(gpu_lib):
    p = configs.abp_config(n=1024, L=16.0, seed=7)
    x, y, th = configs.random_state(p.n, p.L, seed=7)
    with System(p) as s:
        s.upload(x, y, th, step0=123456)
        s.step(20)
        g = s.download()
    assert same(g, O.run32(p, O.State32(x, y, th), 20, step0=123456))


def test_snapshot_resume_is_bitexact(gpu_lib):
    from spp_gb300 import Box
    p = configs.abp_config(n=2048, L=24.0, seed=8)
    x, y, th = configs.random_state(p.n, p.L, seed=8)
    b = Box(p)
    b.Init(x, y, th)
    b.Multi_Step(40)
    snap = b.Save()
    b.Multi_Step(40)
    end1 = b.Save()
    b2 = Box(p)
    b2.Load(snap)
    b2.Multi_Step(40)
    end2 = b2.Save()
    assert np.array_equal(end1.theta, end2.theta) and np.array_equal(end1.x, end2.x)
    assert np.array_equal(end1.img_x, end2.img_x) and np.array_equal(end1.img_y, end2.img_y)
    assert end1.step == end2.step == 80


def test_invalid_inputs_fail_loudly(gpu_lib):
    p = configs.abp_config(n=4, L=4.0)
    with System(p) as s:
        x = np.array([0, 1, 2, 5.0], np.float32)  # outside [-4, 4)
        with pytest.raises(SppError) as e:
            s.upload(x, x, x)
        assert e.value.status == 1
        with pytest.raises(SppError) as e:
            s.upload(np.array([0, 1, np.nan, 0], np.float32), np.zeros(4, np.float32),
                     np.zeros(4, np.float32))
        assert e.value.status == 7
        with pytest.raises(SppError):
            s.step(1)  # nothing uploaded yet
    with pytest.raises(SppError) as e:
        System(configs.abp_config(n=4, L=1.0))
    assert e.value.status == 1


def test_r12_overlap_reports_fixed_point_overflow(gpu_lib):
    p = configs.reference_defaults(abi.MODEL_ABP)
    p.n, p.L, p.dt, p.skin = 2, 4.0, 0.001, 0.3
    x = np.array([0.0, 0.01], np.float32)   # (sigma / d)^13 ~ 1e26
    y = np.zeros(2, np.float32)
    th = np.zeros(2, np.float32)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(1)
        with pytest.raises(SppError) as e:
            s.sync()
        assert e.value.status == 4


def test_kernel_launch_count(gpu_lib):
    p = configs.abp_config(n=4096, L=32.0)
    x, y, th = configs.random_state(p.n, p.L, seed=1)
    with System(p) as s:
        s.upload(x, y, th)
        n0 = s.kernel_launches()
        s.step(64)
        o = s.observables()
        n1 = s.kernel_launches()
    assert n1 - n0 >= 64 * 2


def test_checkpoint_file_resume_is_bitexact(gpu_lib, tmp_path):
    """Checkpoint to a file mid-run, resume in a new system: the continued run
    equals the uninterrupted one bit for bit (Philox counter restored)."""
    from spp_gb300 import checkpoint
    p = configs.abp_config(n=4096, L=32.0, seed=9)
    x, y, th = configs.random_state(p.n, p.L, seed=9)
    path = tmp_path / "ck.npz"
    with System(p) as a:
        a.upload(x, y, th, step0=1000)
        a.step(30)
        checkpoint.save(path, a)
        a.step(45)
        end_a = a.download()
    with checkpoint.resume(path) as b:
        assert b.step0 == 1030
        b.step(45)
        end_b = b.download()
    for u, v in zip(end_a, end_b):
        assert np.array_equal(u, v)


def test_run_and_tumble_checkpoint_resume_is_bitexact(gpu_lib, tmp_path):
    """RTPChain swimmers inside ring membranes, checkpointed mid-run while
    swimmers are tumbling: the tumble state (RTPChain::tumble_flag and
    tumble_elapesed_time, shared/particle.h:1063-1064) is part of the
    checkpoint, so the resumed run equals the uninterrupted one bit for bit,
    through the file and through Box.Save / Box.Load.  Without the tumble
    state the resumed run differs."""
    from spp_gb300 import Box, checkpoint
    p = configs.vesicle_config(n_rings=16, ring_size=64, swimmers_per_ring=16, L=48.0,
                               integrator=abi.INT_RK2, seed=9)
    x, y, th = configs.vesicle_state(p)
    p.rot_noise = abi.NOISE_TUMBLE
    p.tumble_rate, p.tumble_time, p.tumble_torque = 20.0, 0.03, 3.0
    path = tmp_path / "rtp.npz"
    with System(p) as a:
        a.upload(x, y, th)
        a.step(120)
        mid = a.download_tumble()
        checkpoint.save(path, a)
        a.step(80)
        end_a = a.download()
    assert np.count_nonzero(mid) > 0    # swimmers were tumbling at the checkpoint
    with checkpoint.resume(path) as b:
        assert np.array_equal(b.download_tumble(), mid)
        b.step(80)
        end_b = b.download()
    for u, v in zip(end_a, end_b):
        assert np.array_equal(u, v)
    box = Box(p)
    box.Init(x, y, th)
    box.Multi_Step(120)
    snap = box.Save()
    box.Multi_Step(80)
    end_c = box.Save()
    box.Load(snap)
    box.Multi_Step(80)
    end_d = box.Save()
    for u, v in ((end_c.x, end_d.x), (end_c.theta, end_d.theta), (end_c.tumble, end_d.tumble)):
        assert np.array_equal(u, v)
    assert np.array_equal(end_c.x, end_a[0])
    with System(p) as c:       # the same snapshot without its tumble state
        c.upload(snap.x, snap.y, snap.theta, step0=snap.step, img_x=snap.img_x, img_y=snap.img_y)
        c.step(80)
        assert not np.array_equal(c.download()[2], end_a[2])
    with System(p) as d:
        d.upload(x, y, th)
        bad = np.zeros(p.n, np.int32)
        bad[0] = 1                        # particle 0 is a membrane bead: it never tumbles
        with pytest.raises(SppError):
            d.upload_tumble(bad)


def test_densifying_flocks_keep_recovering(gpu_lib):
    """Continuous Vicsek without noise or repulsion: flocks densify, the
    neighbour list overflows again and again as the run goes on; recovery
    keeps growing it, and the run stays bit-exact."""
    p = configs.lyapunov_config(n=1024)
    x, y, th = configs.random_state(p.n, p.L, seed=3)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(1050)
        g = s.download()
        o = s.observables()
    assert o.step == 1050 and o.list_capacity > 16
    assert same(g, O.run32(p, O.State32(x, y, th), 1050))


def test_rejected_upload_then_valid_upload_and_download_into_buffers(gpu_lib):
    """Inputs are checked on the device as they are placed: a bad upload is
    refused (the system holds no state until a good one), and the smallest
    bad index is reported.  Downloads can fill caller buffers."""
    p = configs.abp_config(n=4096, L=32.0, seed=5)
    x, y, th = configs.random_state(p.n, p.L, seed=5)
    bad = x.copy()
    bad[[700, 2000]] = 40.0
    with System(p) as s:
        with pytest.raises(SppError) as e:
            s.upload(bad, y, th)
        assert e.value.status == 1 and "particle 700" in str(e.value)
        with pytest.raises(SppError):
            s.step(1)
        s.upload(x, y, th)
        s.step(10)
        ref = s.download()
        out = tuple(np.empty(p.n, dt) for dt in (np.float32, np.float32, np.float32, np.int32, np.int32))
        got = s.download(out=out)
        assert all(a is b for a, b in zip(got, out))
        for u, v in zip(ref, got):
            assert np.array_equal(u, v)
    assert same(ref, O.run32(p, O.State32(x, y, th), 10))
