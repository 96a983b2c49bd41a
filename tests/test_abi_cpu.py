"""The C-ABI library loads and exports every symbol include/spp.h declares;
entry points that need no GPU answer on the CPU; creating a system without a
GPU fails with a status, not a crash or a silent fallback."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from spp_gb300 import abi, build

HEADER = Path(__file__).resolve().parents[1] / "include" / "spp.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(spp_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return abi.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in abi.PROTOTYPES, f"{n} missing from the ctypes prototypes"


def test_abi_version_and_status_strings(lib):
    assert lib.spp_abi_version() == 1
    assert lib.spp_status_string(0) == b"SPP_OK"
    assert lib.spp_status_string(4) == b"SPP_ERR_OVERFLOW"


def test_params_init_reference_defaults(lib):
    p = abi.SppParams()
    assert lib.spp_params_init(C.byref(p), abi.MODEL_ABP) == 0
    assert p.struct_size == C.sizeof(abi.SppParams)
    assert (p.k_rep, p.sigma_rep, p.r_align, p.r_rep) == (2.0, 1.0, 1.1, 1.2)
    assert p.integrator == abi.INT_RK2 and p.force_law == abi.FORCE_R12_TRUNC
    assert lib.spp_params_init(C.byref(p), 99) == 6


def test_create_rejects_bad_params_without_touching_gpu(lib):
    p = abi.SppParams()
    lib.spp_params_init(C.byref(p), abi.MODEL_ABP)
    h = C.c_void_p()
    bad = p.replace(struct_size=4, n=10)
    assert lib.spp_create(C.byref(bad), C.byref(h)) == abi.SPP_OK + 1
    assert b"struct_size" in lib.spp_last_error()
    assert lib.spp_create(C.byref(p.replace(n=0)), C.byref(h)) == 1
    assert lib.spp_create(C.byref(p.replace(n=10, skin=0.0)), C.byref(h)) == 1
    assert lib.spp_create(C.byref(p.replace(n=10, model=42)), C.byref(h)) == 6
    assert lib.spp_create(C.byref(p.replace(n=10, L=1.0)), C.byref(h)) == 1  # box < 3 cells


def test_create_without_gpu_reports_status(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = abi.SppParams()
    lib.spp_params_init(C.byref(p), abi.MODEL_ABP)
    h = C.c_void_p()
    rc = lib.spp_create(C.byref(p.replace(n=100, L=16.0)), C.byref(h))
    assert rc in (2, 3)  # SPP_ERR_ALLOC / SPP_ERR_CUDA
    assert not h.value


def test_chain_mobility_entry_point(lib):
    """spp_chain_mobility against Set_nb (shared/particle.h:856-876),
    written out here from its formulas."""
    m = np.zeros(3)
    ptr = m.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.spp_chain_mobility(1, 1.0, 1.0, ptr) == 0
    assert list(m) == [0.5, 0.5, 1.0]
    for nb, sep, sig in ((2, 1.0, 1.0), (3, 0.5, 0.5), (8, 0.3, 1.2)):
        assert lib.spp_chain_mobility(nb, sep, sig, ptr) == 0
        ar = 1 / ((sep * (nb - 1) / sig) + 1)
        e2 = 1 - ar * ar
        e = np.sqrt(e2)
        Lg = np.log((1 + e) / (1 - e))
        assert m[0] == 1.0
        assert abs(m[1] - 0.5 * (2 * e + (3 * e2 - 1) * Lg) / ((1 + e2) * Lg - 2 * e)) < 1e-15
        assert abs(m[2] - 6 / (1 + ar * ar) / sig / sig) < 1e-15
        assert 0.5 * m[0] < m[1] < m[0]   # a rod moves more easily along its axis
    assert lib.spp_chain_mobility(9, 1.0, 1.0, ptr) != 0
    assert lib.spp_chain_mobility(2, 0.0, 1.0, ptr) != 0


def test_create_rejects_bad_chains_without_touching_gpu(lib):
    p = abi.SppParams()
    lib.spp_params_init(C.byref(p), abi.MODEL_BEADS)
    assert (p.chain_beads, p.bead_separation, p.sigma_chain, p.r_chain) == (1, 1.0, 1.0, 1.1)
    p.n = 64
    h = C.c_void_p()
    assert lib.spp_create(C.byref(p.replace(chain_beads=9)), C.byref(h)) == 1
    assert lib.spp_create(C.byref(p.replace(chain_beads=-1)), C.byref(h)) == 1
    assert lib.spp_create(C.byref(p.replace(chain_beads=2, bead_separation=0.0)), C.byref(h)) == 1
    assert lib.spp_create(C.byref(p.replace(chain_beads=2, force_law=abi.FORCE_HARMONIC)), C.byref(h)) == 1
    q = abi.SppParams()
    lib.spp_params_init(C.byref(q), abi.MODEL_ABP)
    assert lib.spp_create(C.byref(q.replace(n=64, chain_beads=2)), C.byref(h)) == 6
    assert b"SPP_MODEL_BEADS" in lib.spp_last_error()
