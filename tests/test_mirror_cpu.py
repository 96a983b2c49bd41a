"""The CPU mirror of the kernels' FP32 arithmetic against the FP64 oracle,
and the pair/cell predicates, all on the CPU."""
import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import abi, configs


def wrapped_err(a, b, period):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return np.abs((d + period / 2) % period - period / 2)


def test_mirror_tracks_fp64_abp_short_horizon():
    p = configs.abp_config(n=4096, L=32.0)
    x, y, th = configs.random_state(p.n, p.L, seed=1)
    a = O.run64(p, O.State64(x, y, th), 10)
    b = O.run32(p, O.State32(x, y, th), 10)
    xu = b.x.astype(np.float64) + 2 * p.L * b.ix
    assert np.max(np.abs(xu - a.xu)) / (2 * p.L) < 1e-5
    assert np.max(wrapped_err(b.th, a.th, 2 * np.pi)) < 1e-5


def test_mirror_tracks_fp64_vicsek_short_horizon():
    p = configs.vicsek_config()
    x, y, th = configs.random_state(p.n, p.L, seed=0)
    a = O.run64(p, O.State64(x, y, th), 5)
    b = O.run32(p, O.State32(x, y, th), 5)
    # dt = 1 Vicsek is chaotic: rounding differences of 1e-7 grow by orders of
    # magnitude where a heading sum nearly cancels, so bound quantiles.
    e = wrapped_err(b.th, a.th, 2 * np.pi)
    assert np.median(e) < 1e-6
    assert np.quantile(e, 0.99) < 1e-5
    assert np.max(e) < 1e-2
    assert np.quantile(wrapped_err(b.x, a.x, 2 * p.L), 0.99) < 1e-5


@pytest.mark.parametrize("r", [1.0, 1.3])
def test_pair_sets_fp32_vs_fp64(r):
    p = configs.abp_config(n=4096, L=32.0)
    x, y, _ = configs.random_state(p.n, p.L, seed=3)
    k32 = O.pairs32(p, x, y, r)
    k64 = O.pairs64(x.astype(np.float64), y.astype(np.float64), p.L, r)
    mism = np.setxor1d(k32, k64).size
    # the two predicates may differ only for pairs within rounding of r
    assert mism <= 2, mism
    assert k32.size > 4000


def test_cells_fp32_vs_fp64():
    p = configs.abp_config(n=4096, L=32.0)
    x, y, _ = configs.random_state(p.n, p.L, seed=3)
    for rule in (abi.BIN_GEOMETRIC, abi.BIN_REFERENCE):
        cx, cy = O.cells32(p, x, y, 49, rule)
        dx, dy = O.cells64(x, y, p.L, 49, rule)
        assert np.sum(cx != dx) + np.sum(cy != dy) <= 2


def test_reference_binning_rule_is_integer_aligned():
    """serial/box.h:116-117 casts (x + L) to int before scaling: cells follow
    the integer grid, not the geometric one."""
    p = configs.vicsek_config(n=3, L=4.0)
    x = np.array([-3.9, 0.95, 3.99], np.float32)
    y = np.zeros(3, np.float32)
    cxr, _ = O.cells32(p, x, y, 3, abi.BIN_REFERENCE)
    cxg, _ = O.cells32(p, x, y, 3, abi.BIN_GEOMETRIC)
    # x = 0.95: (int)(4.95) = 4 -> 4*3/8 = 1 ; geometric floor(4.95*3/8) = 1
    assert list(cxr) == [0, 1, 2] and list(cxg) == [0, 1, 2]
    x = np.array([-1.4, -1.1], np.float32)
    y = np.zeros(2, np.float32)
    cxr, _ = O.cells32(p.replace(n=2), x, y, 3, abi.BIN_REFERENCE)
    cxg, _ = O.cells32(p.replace(n=2), x, y, 3, abi.BIN_GEOMETRIC)
    # (int)(2.6) = 2 -> 0.75 -> 0 vs geometric floor(2.6*3/8 = 0.975) = 0; (int)(2.9)=2 -> 0 vs 1.0875 -> 1
    assert list(cxr) == [0, 0] and list(cxg) == [0, 1]


def test_mirror_deterministic_and_polarization():
    p = configs.vicsek_config(n=1024, L=16.0, eta=0.1)
    x, y, th = configs.random_state(p.n, p.L, seed=8)
    a = O.run32(p, O.State32(x, y, th), 60)
    b = O.run32(p, O.State32(x, y, th), 60)
    assert np.array_equal(a.th, b.th)
    P0, _, _ = O.polarization(th)
    P1, _, _ = O.polarization(a.th)
    assert P1 > P0 + 0.2  # low noise orders the flock
