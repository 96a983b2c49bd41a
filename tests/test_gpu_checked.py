"""The bounds-checked build (SPP_CHECKED): every list, cell and slot index the
hot kernels use is checked, an index out of range sets a flag (reported as
SPP_ERR_BOUNDS at the next sync) and the access is skipped.  Built into a
separate library and run through a slice of the parity tests: with the
checks on, the results stay bit-exact and no index is flagged."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.gpu
def test_checked_build_passes_parity(tmp_path):
    env = dict(os.environ)
    env.update(SPP_NVCC_DEFINES="SPP_CHECKED", SPP_LIB_OUT=str(tmp_path / "libspp_checked.so"),
               SPP_BUILD_DIR=str(tmp_path / "build"))
    r = subprocess.run([sys.executable, "-m", "spp_gb300.build", "-f"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    env["SPP_GB300_LIB"] = str(tmp_path / "libspp_checked.so")
    sel = ("abp or vicsek or continuous or long_lists or walls or chains or dimers or "
           "vesicle or run_and_tumble")
    r = subprocess.run([sys.executable, "-m", "pytest", "tests/test_gpu_parity.py", "-m", "gpu", "-q",
                        "-x", "-k", sel, "-p", "no:cacheprovider"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert " passed" in r.stdout
