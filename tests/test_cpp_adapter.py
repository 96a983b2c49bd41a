"""The header-only C++ Box adapter (include/spp_box.hpp) over the C ABI: it
compiles with plain g++ (CPU), and a reference-shaped C++ driver produces the
same bits as the Python path (GPU)."""
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
DRIVER = ROOT / "tests" / "cpp" / "abp_driver.cpp"


def gxx():
    g = shutil.which("g++")
    if g is None:
        pytest.skip("g++ not available")
    return g


def test_adapter_compiles():
    r = subprocess.run([gxx(), "-std=c++14", "-fsyntax-only", "-Wall", "-Wextra",
                        "-I", str(ROOT / "include"), str(DRIVER)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_driver_matches_python(gpu_lib, tmp_path):
    from spp_gb300 import System, configs
    from spp_gb300.abi import LIB_PATH
    libdir = Path(LIB_PATH).parent
    exe = tmp_path / "abp_driver"
    r = subprocess.run([gxx(), "-std=c++14", "-O2", "-I", str(ROOT / "include"), str(DRIVER),
                        "-o", str(exe), "-L", str(libdir), "-lspp_gb300",
                        f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n, L = 2048, 24.0
    x, y, th = configs.random_state(n, L, seed=1)
    state = tmp_path / "state.f32"
    np.concatenate([x, y, th]).astype(np.float32).tofile(state)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(state), str(out), str(n), str(L)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    pol = [float(line.split()[1]) for line in r.stdout.strip().splitlines()]
    assert len(pol) == 4
    raw = out.read_bytes()
    t, Lx, Ly, nb, Ns, Nm = struct.unpack("<dddiii", raw[:36])
    assert (Lx, Ly, nb, Ns, Nm) == (L, L, 1, n, 0) and abs(t - 0.5) < 1e-12
    rec = np.frombuffer(raw[36:], np.float32).reshape(n, 3)
    p = configs.abp_config(n=n, L=L, seed=1)
    with System(p) as s:
        s.upload(x, y, th)
        s.step(100)
        gx, gy, gth, gix, giy = s.download()
        P = s.observables().polarization
    xu = (gx.astype(np.float64) + 2 * L * gix).astype(np.float32)
    assert np.array_equal(rec[:, 0], xu)
    assert np.array_equal(rec[:, 2], gth)
    # the frame reads back through the reference-format reader
    from spp_gb300 import binfile
    (frame,) = binfile.read_frames(raw)
    assert frame.healthy and np.array_equal(frame.x, xu) and np.array_equal(frame.theta, gth)
    assert abs(pol[-1] - P) <= 1e-5 * max(P, 1e-3)  # ostream prints 6 significant digits
