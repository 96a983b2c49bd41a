"""Host side of the launch-shape autotuner: table keys, the persistent table,
argument checks of spp_autotune and of gather_lanes (all answered before any
device work), the ctypes layout of the report, and the CPU mirror honouring
gather_lanes exactly as the automatic rule does."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from spp_gb300 import abi, autotune, build, configs

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    build.build()
    return abi.lib()


def test_table_key_buckets_size_and_density():
    p = configs.abp_config(n=4096, L=32.0)
    k = autotune.table_key(p)
    assert k == autotune.table_key(p.replace(n=4300))            # same octave of N
    assert k != autotune.table_key(p.replace(n=8192))            # next octave
    assert k != autotune.table_key(p.replace(L=32.0 * 2 ** 0.5))  # half the density
    assert k != autotune.table_key(p.replace(skin=0.6))
    assert k != autotune.table_key(p.replace(model=abi.MODEL_CONTINUOUS))
    assert "n2^12" in k and "rho2^+0.0" in k


def test_tuned_params_measures_once_then_reads_the_table(tmp_path):
    p = configs.abp_config(n=2048, L=22.6)
    calls = []

    def fake_measure(q, x, y, th, trial_steps, what):
        calls.append((x.shape, trial_steps, what))
        rows = [{"gather_lanes": 1, "skin": q.skin, "ms_per_step": 0.02, "late_rebuilds": 0,
                 "status": 0, "chosen": False},
                {"gather_lanes": 4, "skin": 2 * q.skin, "ms_per_step": 0.01, "late_rebuilds": 0,
                 "status": 0, "chosen": True}]
        return q.replace(gather_lanes=4, skin=2 * q.skin), rows

    path = tmp_path / "tune.json"
    q = autotune.tuned_params(p, table=autotune.TuneTable(path), trial_steps=50, measure=fake_measure)
    assert len(calls) == 1 and calls[0] == ((2048,), 50, abi.TUNE_LANES | abi.TUNE_SKIN)
    assert (q.gather_lanes, q.skin) == (4, 2 * p.skin)
    assert path.exists()

    def no_measure(*a, **kw):
        raise AssertionError("the table should have answered")

    q2 = autotune.tuned_params(p.replace(n=2100), table=autotune.TuneTable(path), measure=no_measure)
    assert (q2.gather_lanes, q2.skin, q2.n) == (4, 2 * p.skin, 2100)
    # tuning a different set of shapes is a different entry
    autotune.tuned_params(p, table=autotune.TuneTable(path), what=abi.TUNE_SKIN, measure=fake_measure)
    assert len(calls) == 2


def test_autotune_rejects_bad_arguments_before_device_work(lib):
    p = configs.abp_config(n=64, L=8.0)
    x, y, th = (np.zeros(64, np.float32) for _ in range(3))
    f = [a.ctypes.data_as(C.POINTER(C.c_float)) for a in (x, y, th)]
    rep = abi.SppTuneReport()
    both = abi.TUNE_LANES | abi.TUNE_SKIN
    assert lib.spp_autotune(None, f[0], f[1], f[2], 10, both, C.byref(rep)) == 1
    assert lib.spp_autotune(C.byref(p), f[0], f[1], f[2], 10, both, None) == 1
    assert lib.spp_autotune(C.byref(p), f[0], f[1], f[2], 0, both, C.byref(rep)) == 1
    assert b"trial_steps" in lib.spp_last_error()
    assert lib.spp_autotune(C.byref(p), f[0], f[1], f[2], 10, 0, C.byref(rep)) == 1
    assert lib.spp_autotune(C.byref(p), f[0], f[1], f[2], 10, 8, C.byref(rep)) == 1
    v = configs.vicsek_config(n=64, L=8.0)
    assert lib.spp_autotune(C.byref(v), f[0], f[1], f[2], 10, both, C.byref(rep)) == 6


def test_gather_lanes_is_checked_before_device_work(lib):
    h = C.c_void_p()
    p = configs.abp_config(n=64, L=8.0)
    assert lib.spp_create(C.byref(p.replace(gather_lanes=2)), C.byref(h)) == 1
    assert b"gather_lanes" in lib.spp_last_error()
    # multi-bead swimmers keep one thread per body
    chains = configs.chain_config(n=64).replace(gather_lanes=4)
    assert lib.spp_create(C.byref(chains), C.byref(h)) == 6
    vic = configs.vicsek_config(n=64, L=8.0).replace(gather_lanes=4)
    assert lib.spp_create(C.byref(vic), C.byref(h)) == 6


def test_report_layout_matches_the_header():
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "spp.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(SppParams), offsetof(SppParams, gather_lanes),
         sizeof(SppTuneReport), offsetof(SppTuneReport, c[1].skin),
         offsetof(SppTuneReport, c[7].late_rebuilds));
  return 0;
}
'''
    work = Path(build.BUILD)
    work.mkdir(parents=True, exist_ok=True)
    c_file, exe = work / "tune_layout.c", work / "tune_layout"
    c_file.write_text(src)
    subprocess.run([gcc, "-I", str(ROOT / "include"), str(c_file), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    R, Cd = abi.SppTuneReport, abi.SppTuneCandidate
    want = [C.sizeof(abi.SppParams), abi.SppParams.gather_lanes.offset, C.sizeof(R),
            R.c.offset + C.sizeof(Cd) + Cd.skin.offset,
            R.c.offset + 7 * C.sizeof(Cd) + Cd.late_rebuilds.offset]
    assert got == want


@pytest.mark.parametrize("n,L,explicit", [(1024, 16.0, 4), (20000, 70.7, 1)])
def test_mirror_explicit_lanes_equal_the_automatic_rule(n, L, explicit):
    """Automatic lanes are 4 up to 16,384 particles and 1 beyond; naming the
    same count explicitly gives the same bits in the CPU mirror."""
    p = configs.abp_config(n=n, L=L, seed=5)
    x, y, th = configs.random_state(n, L, seed=5)
    a = O.run32(p, O.State32(x, y, th), 8)
    b = O.run32(p.replace(gather_lanes=explicit), O.State32(x, y, th), 8)
    for u, v in ((a.x, b.x), (a.y, b.y), (a.th, b.th)):
        assert np.array_equal(u, v)
