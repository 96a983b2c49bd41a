"""The arithmetic contract (spp_gb300/csrc/spp_fp32.h) on the CPU.

Philox4x32-10 must reproduce the method's published known-answer vectors
(Salmon et al., SC'11; the Random123 distribution's kat_vectors), the numpy
initial-condition generator must agree with the C one, and the FP32
sin/cos/atan2/log/exp must stay within a few ulp of FP64 libm.
"""
import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import configs

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_known_answers(ctr, key, expect):
    assert O.philox(ctr, key) == expect


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_numpy_philox_matches(ctr, key, expect):
    out = configs.philox4x32_10(*[np.array([c], np.uint32) for c in ctr], key[0], key[1])
    assert tuple(int(o[0]) for o in out) == expect


def test_numpy_philox_matches_c_on_many_counters():
    rng = np.random.default_rng(0)
    for _ in range(50):
        ctr = [int(v) for v in rng.integers(0, 2**32, 4)]
        key = [int(v) for v in rng.integers(0, 2**32, 2)]
        out = configs.philox4x32_10(*[np.array([c], np.uint32) for c in ctr], *key)
        assert tuple(int(o[0]) for o in out) == O.philox(ctr, key)


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_round_keys_known_answers(ctr, key, expect):
    """The kernels draw through precomputed round keys (spp_draw_k)."""
    assert O.philox(ctr, key, round_keys=True) == expect


def test_philox_round_keys_match_on_many_counters():
    rng = np.random.default_rng(1)
    for _ in range(200):
        ctr = [int(v) for v in rng.integers(0, 2**32, 4)]
        key = [int(v) for v in rng.integers(0, 2**32, 2)]
        assert O.philox(ctr, key, round_keys=True) == O.philox(ctr, key)


def ulp_err(approx, exact):
    approx = approx.astype(np.float64)
    u = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
    return np.abs(approx - exact) / np.maximum(u, 2.0 ** -149)


def test_sin_cos_accuracy():
    x = np.linspace(-30, 30, 400001).astype(np.float32)
    xd = x.astype(np.float64)
    # absolute error relative to the ulp of 1 near zero crossings
    s = O.math32("sin", x).astype(np.float64)
    c = O.math32("cos", x).astype(np.float64)
    assert np.max(np.abs(s - np.sin(xd))) < 2.5e-7
    assert np.max(np.abs(c - np.cos(xd))) < 2.5e-7
    big = np.abs(np.sin(xd)) > 0.25
    assert np.max(ulp_err(s[big], np.sin(xd[big]))) <= 3.0


def test_atan2_accuracy():
    th = np.linspace(-np.pi, np.pi, 200001)
    r = np.geomspace(1e-3, 1e3, th.size)
    y = (r * np.sin(th)).astype(np.float32)
    x = (r * np.cos(th)).astype(np.float32)
    a = O.math32("atan2", y, x).astype(np.float64)
    e = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.max(np.abs(a - e)) < 5e-7
    assert O.math32("atan2", np.zeros(1), np.zeros(1))[0] == 0.0


def test_log_exp_accuracy():
    u = (np.arange(1, 2**16 + 1) * 2.0**-16).astype(np.float32)
    lg = O.math32("log", u).astype(np.float64)
    ex = np.log(u.astype(np.float64))
    assert np.max(np.abs(lg - ex) / np.maximum(np.abs(ex), 1e-30)[:]) < 5e-7
    x = np.linspace(-20, 20, 100001).astype(np.float32)
    e = O.math32("exp", x).astype(np.float64)
    assert np.max(ulp_err(e, np.exp(x.astype(np.float64)))) <= 3.0


def test_wrap_angle_range():
    th = np.linspace(-50, 50, 100001).astype(np.float32)
    w = O.math32("wrap", th).astype(np.float64)
    assert np.all(w >= -np.pi - 1e-6) and np.all(w <= np.pi + 1e-6)
    assert np.max(np.abs(np.sin(w) - np.sin(th.astype(np.float64)))) < 2e-5


def test_random_state_in_box():
    x, y, th = configs.random_state(10000, 512.0, seed=1)
    assert x.dtype == np.float32
    assert np.all(x >= -512) and np.all(x < 512) and np.all(y >= -512) and np.all(y < 512)
    assert np.all(th >= -np.pi) and np.all(th < np.pi)
    x2, y2, th2 = configs.random_state(10000, 512.0, seed=1)
    assert np.array_equal(x, x2) and np.array_equal(th, th2)
    # a non power-of-two box still lands inside [-L, L)
    x, y, _ = configs.random_state(100000, 13.7, seed=2)
    assert np.all(x < np.float32(13.7)) and np.all(x >= -np.float32(13.7))


def test_fixed_point_sum_is_exact_and_order_independent():
    rng = np.random.default_rng(3)
    for scale in (1e-6, 1e-2, 1.0, 10.0, 3e3):
        x = (rng.standard_normal(300) * scale).astype(np.float32)
        a = O.fx_sum(x)
        for _ in range(5):
            assert O.fx_sum(rng.permutation(x)) == a
        exact = np.sum(np.round(x.astype(np.float64) * 2.0**27)) * 2.0**-27
        units = a[0] * 2**22 + a[1]
        # every term is rounded once to the 2^-27 grid; the integer sum is exact
        assert abs(units * 2.0**-27 - np.sum(x.astype(np.float64))) <= 300 * 2.0**-28 + 1e-12
        assert abs(units * 2.0**-27 - exact) <= 300 * 2.0**-27
        assert abs(a[2] - np.sum(x.astype(np.float64))) <= 1e-6 * max(1.0, abs(a[2])) + 300 * 2.0**-27


def test_rsqrt_within_two_ulp():
    for x in np.geomspace(1e-6, 1e6, 20001).astype(np.float32):
        y = O.rsqrt32(x)
        e = 1.0 / np.sqrt(np.float64(x))
        assert abs(y - e) <= 2.0 * np.spacing(np.float32(e))
