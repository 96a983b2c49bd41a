"""Build recipe for the oracle (test infrastructure only).

- ``oracle/_build/liboracle.so``: the FP64 restatement (spp_oracle64.c) and
  the FP32 kernel-arithmetic mirror (spp_mirror32.c), plain C.
- ``oracle/_ref/libspp_ref.so``: the reference's own shared/particle.h driven
  by ref_harness.cpp, compiled from the reference checkout in place (never
  copied).  Built only where that checkout exists: ``SPP_REFERENCE_DIR``, else
  a directory named ``reference`` beside this repository.

Both use -ffp-contract=off so that only explicit fmaf() calls fuse, exactly as
the kernels (built with -fmad=false) do.
"""
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
REFERENCE_DIR = Path(os.environ.get("SPP_REFERENCE_DIR", str(REPO.parent / "reference")))

CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-Wall",
          "-Wno-unused-function", "-Wno-misleading-indentation"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_oracle(force=False) -> Path:
    out = HERE / "_build" / "liboracle.so"
    srcs = [HERE / "spp_oracle64.c", HERE / "spp_mirror32.c"]
    deps = srcs + [REPO / "include" / "spp.h", REPO / "spp_gb300" / "csrc" / "spp_fp32.h",
                   REPO / "spp_gb300" / "csrc" / "spp_physics.h"]
    if force or _stale(out, deps):
        out.parent.mkdir(parents=True, exist_ok=True)
        _run(["gcc", "-std=gnu11", *CFLAGS, "-pthread", "-o", str(out), *map(str, srcs), "-lm"])
    return out


def build_ref(force=False):
    """Returns the path of the reference harness library, or None where the
    reference checkout is absent."""
    shared = REFERENCE_DIR / "shared"
    out = HERE / "_ref" / "libspp_ref.so"
    if not (shared / "particle.h").exists():
        return out if out.exists() else None
    deps = [HERE / "ref_harness.cpp", HERE / "refshim" / "gsl" / "gsl_rng.h",
            HERE / "refshim" / "gsl" / "gsl_randist.h", shared / "particle.h",
            shared / "vector-set.h", shared / "state-hyper-vector.h",
            REFERENCE_DIR / "analyze" / "statistics.h",
            HERE / "refshim" / "boost" / "algorithm" / "string.hpp",
            REPO / "spp_gb300" / "csrc" / "spp_fp32.h"]
    if force or _stale(out, deps):
        out.parent.mkdir(parents=True, exist_ok=True)
        _run(["g++", "-std=c++14", *CFLAGS, "-w", "-DRUNGE_KUTTA4",
              "-I", str(HERE / "refshim"), "-I", str(shared), "-I", str(REFERENCE_DIR / "analyze"),
              "-o", str(out), str(HERE / "ref_harness.cpp"), "-lm"])
    return out


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
