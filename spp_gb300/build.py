"""Build the sm_103a CUDA library in-tree: spp_gb300/lib/libspp_gb300.so.

Each .cu under csrc/ compiles in parallel with
  nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -fmad=false
-fmad=false keeps every multiply and add separately rounded unless the
source writes fmaf(), which is what lets the CPU mirror reproduce the
kernels' bits.  The objects link into one shared library with a static
CUDA runtime, so the library carries no dependency beyond the driver.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
# SPP_LIB_OUT / SPP_BUILD_DIR / SPP_NVCC_DEFINES let a launch-shape sweep build
# variants side by side (e.g. SPP_NVCC_DEFINES="SPP_STAGE_MIN_BLOCKS=8").
OUT = Path(os.environ.get("SPP_LIB_OUT", PKG / "lib" / "libspp_gb300.so"))
BUILD = Path(os.environ.get("SPP_BUILD_DIR", PKG / "_build"))
DEFINES = [f"-D{d}" for d in os.environ.get("SPP_NVCC_DEFINES", "").split() if d]

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-ffp-contract=off", "-I", str(PKG.parent / "include")]


def sources():
    return sorted(CSRC.glob("*.cu"))


def headers():
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "spp.h"]


def _stale(out, deps):
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src, extra):
    obj = BUILD / (src.stem + ".o")
    deps = [src] + headers()
    if _stale(obj, deps):
        cmd = [NVCC, *ARCH, *FLAGS, *DEFINES, *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.stderr.strip() and "-Xptxas" in " ".join(extra):
            print(r.stderr, file=sys.stderr)
    return obj


def build(force=False, verbose_ptxas=False):
    BUILD.mkdir(parents=True, exist_ok=True)
    OUT.parent.mkdir(parents=True, exist_ok=True)
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if force or _stale(OUT, objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", str(OUT), *map(str, objs), "-lcudart_static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build(force="-f" in sys.argv, verbose_ptxas="-v" in sys.argv))
