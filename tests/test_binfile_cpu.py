"""The .bin trajectory format (reference writer parallel/box.h:476-502,
reader analyze/read.h:215-270): byte layout, round trips, membranes, and the
reader's health rules."""
import struct

import numpy as np
import pytest

from spp_gb300 import abi, binfile, configs


def test_header_and_record_layout():
    x = np.array([1.5, -2.25], np.float32)
    y = np.array([0.5, 3.0], np.float32)
    th = np.array([0.1, -3.0], np.float32)
    raw = binfile.encode_frame(12.5, 32.0, x, y, th)
    # field by field as the reference writes them: t, Lx, Ly (f64), nb, Ns, Nm (i32),
    # then per swimmer x, y, theta (f32)
    expect = struct.pack("<dddiii", 12.5, 32.0, 32.0, 1, 2, 0) + struct.pack(
        "<ffffff", 1.5, 0.5, np.float32(0.1), -2.25, 3.0, -3.0)
    assert raw == expect


def test_round_trip_with_membrane():
    rng = np.random.default_rng(1)
    frames = []
    for k in range(3):
        x, y, th = (rng.standard_normal(5).astype(np.float32) for _ in range(3))
        mx, my = (rng.standard_normal(4).astype(np.float32) for _ in range(2))
        frames.append((k * 0.5, x, y, th, mx, my))
    raw = b"".join(binfile.encode_frame(t, 10.0, x, y, th, mx, my) for t, x, y, th, mx, my in frames)
    out = binfile.read_frames(raw)
    assert len(out) == 3
    for f, (t, x, y, th, mx, my) in zip(out, frames):
        assert f.healthy and f.t == t and f.Lx == 10.0 and f.nb == 1
        for a, b in ((f.x, x), (f.y, y), (f.theta, th), (f.mx, mx), (f.my, my)):
            assert np.array_equal(a, b)


def test_reader_health_rules():
    x = np.zeros(3, np.float32)
    good = binfile.encode_frame(1.0, 5.0, x, x, x)
    bad_t = binfile.encode_frame(-1.0, 5.0, x, x, x)
    frames = binfile.read_frames(good + bad_t + good + good[:-4])
    # the truncated last frame ends the list; t < 0 marks a frame unhealthy
    assert [f.healthy for f in frames] == [True, False, True]


def test_state_frame_unwraps_and_splits_membrane():
    p = configs.vesicle_config(n_rings=4, ring_size=16, swimmers_per_ring=2)
    n = p.n
    nm = p.n_rings * p.ring_size
    rng = np.random.default_rng(2)
    x = rng.uniform(-p.L, p.L, n).astype(np.float32)
    y = rng.uniform(-p.L, p.L, n).astype(np.float32)
    th = rng.uniform(-3, 3, n).astype(np.float32)
    ix = rng.integers(-2, 3, n).astype(np.int32)
    iy = rng.integers(-2, 3, n).astype(np.int32)
    (f,) = binfile.read_frames(binfile.state_frame(p, 3.0, x, y, th, ix, iy))
    assert len(f.mx) == nm and len(f.x) == n - nm
    xu = (x.astype(np.float64) + 2 * p.L * ix).astype(np.float32)
    assert np.array_equal(f.mx, xu[:nm]) and np.array_equal(f.x, xu[nm:])
    assert np.array_equal(f.theta, th[nm:])


def test_checkpoint_file_format(tmp_path):
    import ctypes as C

    import pytest

    from spp_gb300 import checkpoint
    p = configs.abp_config(n=8, L=4.0, seed=3)
    p.struct_size = C.sizeof(abi.SppParams)
    p.gather_lanes = 4   # a tuned lane count is part of the result and travels with the state
    raw = bytes(C.string_at(C.addressof(p), C.sizeof(p)))
    x = np.arange(8, dtype=np.float32)
    path = tmp_path / "ck.npz"
    np.savez(path, format=checkpoint.FORMAT, params=np.frombuffer(raw, np.uint8), x=x, y=-x, theta=x / 8,
             img_x=np.ones(8, np.int32), img_y=np.zeros(8, np.int32), step=np.int64(77))
    q, snap = checkpoint.load(path)
    assert bytes(q) == raw and snap.step == 77 and np.array_equal(snap.y, -x)
    assert q.gather_lanes == 4
    # a record of the layout before the chain fields (struct_size 240)
    old = bytearray(raw[:240])
    old[:4] = (240).to_bytes(4, "little")
    np.savez(path, format=checkpoint.FORMAT, params=np.frombuffer(bytes(old), np.uint8), x=x, y=-x,
             theta=x / 8, img_x=np.ones(8, np.int32), img_y=np.zeros(8, np.int32), step=np.int64(5))
    q, _ = checkpoint.load(path)
    assert q.struct_size == C.sizeof(abi.SppParams) and q.chain_beads == 0 and q.L == p.L
    old[:4] = (200).to_bytes(4, "little")
    np.savez(path, format=checkpoint.FORMAT, params=np.frombuffer(bytes(old), np.uint8), x=x, y=-x,
             theta=x / 8, img_x=np.ones(8, np.int32), img_y=np.zeros(8, np.int32), step=np.int64(5))
    with pytest.raises(ValueError):
        checkpoint.load(path)
    np.savez(path, format=99, params=np.frombuffer(raw, np.uint8))
    with pytest.raises(ValueError):
        checkpoint.load(path)


def test_chain_frames_carry_chain_length():
    """The header's nb is the first swimmer's chain length (parallel/box.h:485)."""
    p = configs.chain_config(n=9, chain_beads=3)
    x, y, th = configs.chain_state(p)
    z = np.zeros(9, np.int32)
    f = binfile.read_frames(binfile.state_frame(p, 0.5, x, y, th, z, z))[0]
    assert f.nb == 3 and len(f.x) == 9 and len(f.mx) == 0
    q = configs.vesicle_config(n_rings=2, ring_size=40, swimmers_per_ring=1, L=20.0)
    xv, yv, tv = configs.vesicle_state(q)
    z = np.zeros(q.n, np.int32)
    assert binfile.read_frames(binfile.state_frame(q, 0.0, xv, yv, tv, z, z))[0].nb == 1


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_records_match_the_reference_writer(kind):
    """Where the reference checkout is present, the frame's particle records
    are byte for byte what the reference's own Write methods emit
    (shared/particle.h compiled in the oracle harness): kind 0
    RepulsiveParticle::Write (:759-764, x, y, theta), kind 1 a membrane bead
    of ActiveBrownianChain::Write (F0 = 0, :1038-1039, x, y), kind 2 one of
    its swimmers (:1040-1045).  Values include large unwrapped positions and
    the float32 rounding edge."""
    import ctypes as C
    from oracle import oracle as O
    r = O.ref()
    if r is None:
        pytest.skip("reference checkout absent")
    rng = np.random.default_rng(kind)
    n = 300
    xu = np.concatenate([rng.uniform(-5e4, 5e4, n - 4), [0.0, -0.0, 1.0 + 2.0 ** -24, 16777217.0]])
    yu = rng.uniform(-5e4, 5e4, n)
    th = rng.uniform(-np.pi, np.pi, n)
    buf = C.create_string_buffer(16 * n)
    m = r.ref_write_records(kind, n, O._d(xu), O._d(yu), O._d(th), buf, 16 * n)
    assert m == (8 if kind == 1 else 12) * n
    frame = binfile.encode_frame(1.5, 64.0, xu, yu, th) if kind != 1 else \
        binfile.encode_frame(1.5, 64.0, [], [], [], mx=xu, my=yu)
    assert frame[binfile.HEADER.size:] == buf.raw[:m]


def test_records_match_the_reference_fixture():
    """The same pin replayed from tests/golden/reference_records.npz (made by
    tests/golden/make_golden.py from the reference's Write methods)."""
    from pathlib import Path
    z = np.load(Path(__file__).resolve().parent / "golden" / "reference_records.npz")
    xu, yu, th = z["xu"], z["yu"], z["theta"]
    head = binfile.HEADER.size
    assert binfile.encode_frame(0.0, 8.0, xu, yu, th)[head:] == z["kind0"].tobytes()
    assert binfile.encode_frame(0.0, 8.0, xu, yu, th)[head:] == z["kind2"].tobytes()
    assert binfile.encode_frame(0.0, 8.0, [], [], [], mx=xu, my=yu)[head:] == z["kind1"].tobytes()
