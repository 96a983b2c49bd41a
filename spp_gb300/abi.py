"""ctypes mirror of include/spp.h and the loader of the CUDA library.

The product path is ``spp_gb300/lib/libspp_gb300.so`` (hand-written sm_103a
kernels behind the C ABI).  There is no CPU fallback: if the library is
missing, :func:`lib` raises.
"""
import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libspp_gb300.so"

SPP_OK = 0
STATUS_NAMES = {0: "SPP_OK", 1: "SPP_ERR_INVALID", 2: "SPP_ERR_ALLOC", 3: "SPP_ERR_CUDA",
                4: "SPP_ERR_OVERFLOW", 5: "SPP_ERR_TIMEOUT", 6: "SPP_ERR_UNSUPPORTED",
                7: "SPP_ERR_NUMERIC", 8: "SPP_ERR_BOUNDS"}

MODEL_VICSEK, MODEL_VICSEK_REF_ANGLE, MODEL_VICSEK_REF_VECTOR = 0, 1, 2
MODEL_CONTINUOUS, MODEL_ABP, MODEL_BEADS = 3, 4, 5
NOISE_GAUSSIAN, NOISE_TUMBLE = 0, 1
BOUNDARY_PERIODIC, BOUNDARY_WALLS, BOUNDARY_CIRCLE = 0, 1, 2
INT_EULER, INT_RK2, INT_RK4 = 1, 2, 4
FORCE_NONE, FORCE_HARMONIC, FORCE_R12_TRUNC = 0, 1, 2
ALIGN_REFERENCE, ALIGN_MEAN = 0, 1
BIN_GEOMETRIC, BIN_REFERENCE = 0, 1


class SppParams(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("model", C.c_int32), ("integrator", C.c_int32),
        ("force_law", C.c_int32), ("align_mode", C.c_int32), ("n", C.c_int32),
        ("seed", C.c_uint64), ("system_id", C.c_uint32), ("n_rings", C.c_int32),
        ("ring_size", C.c_int32), ("list_capacity", C.c_int32),
        ("L", C.c_double), ("dt", C.c_double), ("v0", C.c_double), ("Dr", C.c_double),
        ("eta", C.c_double), ("g", C.c_double), ("alpha", C.c_double), ("r_align", C.c_double),
        ("r_rep", C.c_double), ("k_rep", C.c_double), ("sigma_rep", C.c_double),
        ("skin", C.c_double), ("beta_push", C.c_double), ("r_push", C.c_double),
        ("mu", C.c_double), ("k_perp", C.c_double), ("torque0", C.c_double),
        ("k_bond", C.c_double), ("bond_rest", C.c_double), ("kappa_bend", C.c_double), ("rot_noise", C.c_int32), ("gather_lanes", C.c_int32),
        ("tumble_rate", C.c_double), ("tumble_time", C.c_double), ("tumble_torque", C.c_double),
        ("chain_beads", C.c_int32), ("reserved2", C.c_int32),
        ("bead_separation", C.c_double), ("sigma_chain", C.c_double), ("r_chain", C.c_double),
        ("boundary", C.c_int32), ("n_walls", C.c_int32), ("walls", (C.c_double * 4) * 4),
        ("A_w", C.c_double), ("sigma_w", C.c_double), ("r_c_w", C.c_double), ("r_f_w", C.c_double),
        ("g_w", C.c_double), ("g_w_cont", C.c_double),
    ]

    def copy(self):
        q = SppParams()
        C.pointer(q)[0] = self
        return q

    def replace(self, **kw):
        q = self.copy()
        for k, v in kw.items():
            set_field(q, k, v)
        return q

    def as_dict(self):
        def plain(v):
            return [plain(e) for e in v] if isinstance(v, C.Array) else v
        return {name: plain(getattr(self, name)) for name, _ in self._fields_}


class SppObservables(C.Structure):
    _fields_ = [
        ("step", C.c_int64), ("t", C.c_double), ("px", C.c_double), ("py", C.c_double),
        ("polarization", C.c_double), ("n_rebuilds", C.c_int64), ("n", C.c_int32),
        ("list_capacity", C.c_int32), ("max_neighbors", C.c_int32), ("cells_per_side", C.c_int32),
        ("late_rebuilds", C.c_int64), ("list_regrowths", C.c_int64), ("bulk_timeouts", C.c_int64),
    ]


class SppRingMotion(C.Structure):
    _fields_ = [(f, C.c_double) for f in ("mb_v_cm_x", "mb_v_cm_y", "mb_l", "mb_omega", "sw_v_cm_x",
                                          "sw_v_cm_y", "sw_l", "sw_omega", "sw_spin")]


class SppProfile(C.Structure):
    _fields_ = [("steps", C.c_int64), ("stage_launches", C.c_int64), ("stage_ms", C.c_double),
                ("rebuilds", C.c_int64), ("rebuild_ms", C.c_double), ("total_ms", C.c_double)]


class SppSweepStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("active", C.c_int32), ("reserved", C.c_int32),
                ("window_steps", C.c_int64), ("p_mean", C.c_double), ("p_var", C.c_double),
                ("p_kurt", C.c_double), ("stationary_steps", C.c_int64),
                ("p_stationary", C.c_double), ("p2_stationary", C.c_double),
                ("p_last", C.c_double), ("p4_stationary", C.c_double), ("binder", C.c_double),
                ("binder_reference", C.c_double)]


class SppRingShape(C.Structure):
    _fields_ = [(f"{pre}_{k}", C.c_double) for pre in ("mb", "sw")
                for k in ("cm_x", "cm_y", "xx", "yy", "xy", "lambda1", "lambda2", "Rg", "Delta")]


class SppOrderStats(C.Structure):
    _fields_ = [("samples", C.c_int64), ("mean", C.c_double), ("mean_square", C.c_double),
                ("variance", C.c_double), ("std", C.c_double), ("min", C.c_double), ("max", C.c_double),
                ("corr_len", C.c_double), ("error", C.c_double), ("sigma2", C.c_double),
                ("p4_mean", C.c_double), ("binder", C.c_double), ("binder_reference", C.c_double)]


TUNE_LANES, TUNE_SKIN = 1, 2
TUNE_MAX_CANDIDATES = 8


class SppTuneCandidate(C.Structure):
    _fields_ = [("gather_lanes", C.c_int32), ("status", C.c_int32), ("skin", C.c_double),
                ("ms_per_step", C.c_double), ("late_rebuilds", C.c_int64)]


class SppTuneReport(C.Structure):
    _fields_ = [("n_candidates", C.c_int32), ("best", C.c_int32),
                ("c", SppTuneCandidate * TUNE_MAX_CANDIDATES)]


def set_field(p, name, value):
    """Sets a field, array fields (walls) from nested sequences.  "reserved"
    is the former name of gather_lanes (0 in parameter records written
    before it had a meaning, i.e. the automatic lane count)."""
    if name == "reserved":
        name = "gather_lanes"
    cur = getattr(p, name)
    if isinstance(cur, C.Array):
        for a, row in enumerate(value):
            for b, v in enumerate(row):
                cur[a][b] = v
    else:
        setattr(p, name, value)


def new_params(**kw) -> SppParams:
    p = SppParams()
    p.struct_size = C.sizeof(SppParams)
    for k, v in kw.items():
        set_field(p, k, v)
    return p


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_I32 = C.POINTER(C.c_int32)
_D = C.POINTER(C.c_double)
_U64 = C.POINTER(C.c_uint64)

# name -> (restype, argtypes); every entry point declared in include/spp.h
PROTOTYPES = {
    "spp_abi_version": (C.c_int, []),
    "spp_status_string": (C.c_char_p, [C.c_int]),
    "spp_last_error": (C.c_char_p, []),
    "spp_params_init": (C.c_int, [C.POINTER(SppParams), C.c_int]),
    "spp_chain_mobility": (C.c_int, [C.c_int, C.c_double, C.c_double, _D]),
    "spp_create": (C.c_int, [C.POINTER(SppParams), C.POINTER(_P)]),
    "spp_destroy": (C.c_int, [_P]),
    "spp_set_stream": (C.c_int, [_P, _P]),
    "spp_upload_state": (C.c_int, [_P, _F, _F, _F, _I32, _I32, C.c_int, C.c_int64]),
    "spp_download_state": (C.c_int, [_P, _F, _F, _F, _I32, _I32, C.c_int]),
    "spp_download_tumble": (C.c_int, [_P, C.POINTER(C.c_int32), C.c_int]),
    "spp_upload_tumble": (C.c_int, [_P, C.POINTER(C.c_int32), C.c_int]),
    "spp_step": (C.c_int, [_P, C.c_int]),
    "spp_sync": (C.c_int, [_P]),
    "spp_observables": (C.c_int, [_P, C.POINTER(SppObservables)]),
    "spp_pairs": (C.c_int, [_P, C.c_double, _I32, _I32, C.c_int, C.POINTER(C.c_int64)]),
    "spp_cells": (C.c_int, [_P, C.c_int, C.c_int, _I32, _I32, C.c_int]),
    "spp_kernel_launches": (C.c_int64, [_P]),
    "spp_stream": (_P, [_P]),
    "spp_profile": (C.c_int, [_P, C.c_int, C.POINTER(SppProfile)]),
    "spp_time_steps": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double)]),
    "spp_batch_create": (C.c_int, [C.POINTER(SppParams), C.c_int, C.POINTER(_P)]),
    "spp_batch_destroy": (C.c_int, [_P]),
    "spp_batch_set_windows": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "spp_batch_upload": (C.c_int, [_P, _F, _F, _F, C.c_int]),
    "spp_batch_step": (C.c_int, [_P, C.c_int]),
    "spp_batch_poll": (C.c_int, [_P, C.POINTER(SppSweepStats), C.c_int]),
    "spp_batch_retire": (C.c_int, [_P, _I32, C.c_int]),
    "spp_batch_resume": (C.c_int, [_P, _I32, C.c_int]),
    "spp_batch_download": (C.c_int, [_P, _F, _F, _F, _I32, _I32, C.c_int]),
    "spp_batch_kernel_launches": (C.c_int64, [_P]),
    "spp_batch_time_steps": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double)]),
    "spp_order_parameters": (C.c_int, [_D, C.c_int, C.c_double, C.POINTER(SppOrderStats)]),
    "spp_polarization_series": (C.c_int, [_P, C.c_int, C.c_int, _D, _D, _D]),
    "spp_radial_distribution": (C.c_int, [_P, C.c_double, C.c_int, _U64]),
    "spp_pair_distribution": (C.c_int, [_P, C.c_double, C.c_double, C.c_int, C.c_int, _U64]),
    "spp_ring_shapes": (C.c_int, [_P, C.POINTER(SppRingShape), C.c_int]),
    "spp_ring_motion_mark": (C.c_int, [_P]),
    "spp_ring_motion": (C.c_int, [_P, C.c_void_p, C.c_int]),
    "spp_mlp_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(_P)]),
    "spp_mlp_destroy": (C.c_int, [_P]),
    "spp_mlp_num_params": (C.c_int, [_P]),
    "spp_mlp_set_params": (C.c_int, [_P, _F]),
    "spp_mlp_get_params": (C.c_int, [_P, _F]),
    "spp_mlp_predict": (C.c_int, [_P, _F, C.c_int, _F]),
    "spp_mlp_grad": (C.c_int, [_P, _F, _F, _F, C.c_int, _F, _F]),
    "spp_mlp_train": (C.c_int, [_P, _F, _F, _F, C.c_int, C.c_int, C.c_float, _F]),
    "spp_lyap_init": (C.c_int, [_P, C.c_int, C.c_uint64]),
    "spp_lyap_set_vectors": (C.c_int, [_P, _F, C.c_int]),
    "spp_lyap_step": (C.c_int, [_P, C.c_int, C.c_int]),
    "spp_lyap_exponents": (C.c_int, [_P, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double)]),
    "spp_lyap_vectors": (C.c_int, [_P, _F, C.c_int]),
    "spp_pairs_noalloc": (C.c_int, [_P, _P, C.c_int, C.c_double, C.c_double, _P, _P, C.c_int64,
                                    _P, _P]),
    "spp_autotune": (C.c_int, [C.POINTER(SppParams), _F, _F, _F, C.c_int, C.c_int,
                               C.POINTER(SppTuneReport)]),
}

_lib = None


def lib():
    """Load the CUDA library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("SPP_GB300_LIB", LIB_PATH))
        if not path.exists():
            raise RuntimeError(
                f"{path} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(str(path))
        for name, (res, args) in PROTOTYPES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class SppError(RuntimeError):
    def __init__(self, status, where):
        msg = ""
        try:
            msg = lib().spp_last_error().decode()
        except Exception:
            pass
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {msg}")
        self.status = status


def check(status, where):
    if status != SPP_OK:
        raise SppError(status, where)
    return status


def fptr(a):
    return a.ctypes.data_as(_F) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_I32) if a is not None else None
