"""Order-parameter statistics (host code of the library) against the FP64
restatement of the reference's Stat / Compute_Order_Parameters, and the
FP32 mirror of the pair histograms against the FP64 restatement of
Pair_Distribution and a radial histogram.  No GPU: spp_order_parameters
makes no CUDA call."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import analysis_oracle as A
from oracle import oracle as O
from spp_gb300 import abi, observables


def ar1(T, phi, seed, mean=0.6, sd=0.05):
    rng = np.random.default_rng(seed)
    x = np.empty(T)
    x[0] = mean
    for t in range(1, T):
        x[t] = mean + phi * (x[t - 1] - mean) + sd * rng.standard_normal()
    return x


@pytest.mark.parametrize("T,phi,seed", [(600, 0.9, 1), (1000, 0.0, 2), (257, 0.98, 3), (2, 0.5, 4)])
def test_order_parameters_bitexact_vs_restatement(T, phi, seed):
    p = ar1(T, phi, seed)
    got = observables.order_parameters(p, area=4096.0)
    ref = A.order_parameters(list(p), 4096.0)
    for key in ("mean", "mean_square", "variance", "std", "min", "max", "corr_len", "error", "sigma2",
                "p4_mean", "binder", "binder_reference"):
        assert got[key] == ref[key], key
    assert got["samples"] == T


def test_correlated_series_has_longer_correlation_and_larger_error():
    slow = observables.order_parameters(ar1(4000, 0.95, 5), 1.0)
    fast = observables.order_parameters(ar1(4000, 0.0, 5), 1.0)
    assert slow["corr_len"] > 10 * max(fast["corr_len"], 1.0)
    # error = sqrt(var * corr_len / T): the naive sqrt(var / T) underestimates it
    assert slow["error"] > 3 * math.sqrt(slow["variance"] / 4000)


def test_binder_forms_on_a_constant_series():
    got = observables.order_parameters(np.full(50, 0.5), 1.0)
    # standard form: 1 - P^4 / (3 P^4) = 2/3; the reference's: 1 - P^4 / (3 P^2)
    assert got["binder"] == pytest.approx(2.0 / 3.0)
    assert got["binder_reference"] == pytest.approx(1 - 0.0625 / 0.75)
    # zero variance: the autocorrelation is 0/0 and never falls below 0.01,
    # so the reference's loop runs to T/2 - 1 and the error is 0
    assert got["corr_len"] == 24 and got["error"] == 0.0


def test_order_parameters_rejects_bad_input():
    with pytest.raises(abi.SppError):
        observables.order_parameters(np.array([0.5]), 1.0)
    with pytest.raises(abi.SppError):
        observables.order_parameters(np.array([0.5, np.nan, 0.1]), 1.0)


def test_radial_histogram_mirror_vs_fp64():
    rng = np.random.default_rng(7)
    L = 8.0
    x = rng.uniform(-L, L, 300).astype(np.float32)
    y = rng.uniform(-L, L, 300).astype(np.float32)
    h32 = O.radial32(x, y, L, 4.0, 40).astype(np.int64)
    h64 = A.radial_counts(x, y, L, 4.0, 40)
    # FP32 and FP64 distances may fall on either side of a bin edge
    assert np.abs(h32 - h64).sum() <= 4
    assert h32.sum() % 2 == 0  # ordered pairs: each unordered pair twice


def test_pair_distribution_mirror_vs_fp64():
    rng = np.random.default_rng(8)
    L = 8.0
    x = rng.uniform(-L, L, 300).astype(np.float32)
    y = rng.uniform(-L, L, 300).astype(np.float32)
    th = rng.uniform(-np.pi, np.pi, 300).astype(np.float32)
    c, s = O.math32("cos", th), O.math32("sin", th)
    h32 = O.pair_distribution32(x, y, c, s, 2.0, 3.0, 12, 18).astype(np.int64)
    h64 = A.pair_distribution(x, y, th, 2.0, 3.0, 12, 18)
    assert abs(int(h32.sum()) - int(h64.sum())) <= 2
    assert np.abs(h32 - h64).sum() <= 6


def test_g_of_r_of_uniform_points_is_near_one():
    rng = np.random.default_rng(9)
    L = 10.0
    n = 2000
    x = rng.uniform(-L, L, n).astype(np.float32)
    y = rng.uniform(-L, L, n).astype(np.float32)
    r, g = observables.radial_g(O.radial32(x, y, L, 3.0, 10), n, L, 3.0)
    assert np.all(np.abs(g[2:] - 1) < 0.1)


ORDER_GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_order_parameters.npz"


def test_order_parameters_bitexact_vs_reference_fixtures():
    """The library's statistics equal the reference's own Stat::Compute,
    Find_Correlation_Length (analyze/statistics.h:35-82) and the combination
    of Compute_Order_Parameters (analyze/analyze.h:121-146), compiled
    unmodified in the oracle harness, bit for bit: fixtures made by
    tests/golden/make_golden.py, replayed everywhere."""
    z = np.load(ORDER_GOLDEN)
    keys = json.loads(bytes(z["keys"]).decode())
    cases = sorted({k.split("/")[0] for k in z.files if "/" in k})
    assert len(cases) == 5
    for case in cases:
        got = observables.order_parameters(z[f"{case}/in"], area=4096.0)
        for key, want in zip(keys, z[f"{case}/out"]):
            assert got[key] == want, (case, key)


def test_order_parameters_bitexact_vs_reference_live():
    """Where the reference checkout is present: the same on fresh series,
    and the fixtures are what the reference produces today."""
    r = O.ref()
    if r is None:
        pytest.skip("reference checkout absent; the fixtures pin the statistics instead")
    keys = ["mean", "mean_square", "variance", "std", "min", "max", "corr_len", "error", "sigma2",
            "p4_mean", "binder_reference"]
    for T, phi, seed in [(800, 0.95, 11), (3, 0.0, 12), (4000, 0.999, 13)]:
        x = ar1(T, phi, seed)
        out = np.zeros(len(keys))
        assert r.ref_order_parameters(O._d(x), T, 1024.0, O._d(out)) == 0
        got = observables.order_parameters(x, area=1024.0)
        for key, want in zip(keys, out):
            assert got[key] == want, (T, key)
    z = np.load(ORDER_GOLDEN)
    for case in sorted({k.split("/")[0] for k in z.files if "/" in k}):
        x = z[f"{case}/in"]
        out = np.zeros(len(keys))
        assert r.ref_order_parameters(O._d(x), len(x), 4096.0, O._d(out)) == 0
        assert np.array_equal(out, z[f"{case}/out"]), case
