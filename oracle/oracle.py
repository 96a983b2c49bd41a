"""ctypes front of the oracle libraries -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker.  Nothing in spp_gb300/ imports it.
"""
import ctypes as C
from pathlib import Path

import numpy as np

from spp_gb300 import abi

from . import build as _build

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_U64 = C.POINTER(C.c_uint64)
_P = C.POINTER(abi.SppParams)

_orc = None
_ref = None


def orc():
    global _orc
    if _orc is None:
        L = C.CDLL(str(_build.build_oracle()))
        L.orc64_run.argtypes = [_P, C.c_int, C.c_int64, _D, _D, _D, _D, _D]
        L.orc64_run.restype = C.c_int
        L.orc64_pairs.argtypes = [C.c_int, _D, _D, C.c_double, C.c_double, _I, _I, C.c_int64]
        L.orc64_pairs.restype = C.c_int64
        L.orc_cells.argtypes = [C.c_int, _D, _D, C.c_double, C.c_int, C.c_int, _I, _I]
        L.orc_polarization.argtypes = [C.c_int, _D, _D, _D]
        L.orc_polarization.restype = C.c_double
        L.orc32_run.argtypes = [_P, C.c_int, C.c_int64, _F, _F, _F, _I, _I]
        L.orc32_run.restype = C.c_int
        L.orc32_pairs.argtypes = [_P, _F, _F, C.c_double, _I, _I, C.c_int64]
        L.orc32_pairs.restype = C.c_int64
        L.orc32_cells.argtypes = [_P, _F, _F, C.c_int, C.c_int, _I, _I]
        L.orc32_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc32_philox_ks.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc32_math.argtypes = [C.c_int, C.c_int, _F, _F, _F]
        L.orc32_fx_sum.argtypes = [C.c_int, _F, _I, _I, _F]
        L.orc32_renormalize.argtypes = [C.c_int, C.c_int, _F, _D, C.c_int]
        L.orc32_lyap_init.argtypes = [_P, C.c_int, C.c_uint64, _F]
        L.orc32_lyap_run.argtypes = [_P, C.c_int, C.c_int64, C.c_int, C.c_int, _F, _F, _F, _I, _I,
                                     _F, _D]
        L.orc64_lyap_tangent.argtypes = [_P, C.c_int, C.c_int, C.c_int, _D, _D, _D, _D, _D, _D, _D]
        L.orc64_lyap_clone.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_double, _D, _D, _D, _D,
                                       _D, _D, _D]
        L.orc64_gram_schmidt.argtypes = [C.c_int, C.c_int, _D, _D, C.c_double]
        L.orc32_rsqrt.argtypes = [C.c_float]
        L.orc32_wall_terms.argtypes = [_P, C.c_float, C.c_float, C.c_float, _F]
        L.orc32_wall_terms.restype = None
        L.orc64_wall_terms.argtypes = [_P, C.c_double, C.c_double, C.c_double, _D]
        L.orc64_wall_terms.restype = None
        L.orc32_tumble_steps.argtypes = [_P]
        L.orc32_tumble_steps.restype = C.c_int32
        L.orc32_radial.argtypes = [_F, _F, C.c_int, C.c_double, C.c_double, C.c_int, _U64, C.c_int]
        L.orc32_pair_distribution.argtypes = [_F, _F, _F, _F, C.c_int, C.c_double, C.c_double, C.c_int,
                                              C.c_int, _U64]
        L.orc32_rsqrt.restype = C.c_float
        L.orc32_circle_torque.argtypes = [_P, C.c_float, C.c_float, C.c_float]
        L.orc32_circle_torque.restype = C.c_float
        _I8 = C.POINTER(C.c_int8)
        for nm in ("orc64_watch", "orc32_watch"):
            f = getattr(L, nm)
            f.argtypes = [_I, _I, _I, _I8, _D, C.c_int64, C.c_double, C.c_double]
            f.restype = None
        for nm in ("orc64_watch_count", "orc32_watch_count"):
            getattr(L, nm).restype = C.c_int64
        _orc = L
    return _orc


def ref():
    """The reference-harness library, or None where the reference is absent."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None or not Path(path).exists():
            return None
        L = C.CDLL(str(path))
        L.ref_run.argtypes = [_P, C.c_int, C.c_int64, _D, _D, _D, _D, _D]
        L.ref_run.restype = C.c_int
        L.ref_wall_terms.argtypes = [_P, C.c_double, C.c_double, C.c_double, _D]
        L.ref_wall_terms.restype = None
        L.ref_r12_truncated.argtypes = [C.c_double] * 5 + [_D, _D]
        L.ref_spring.argtypes = [C.c_double] * 4 + [_D, _D]
        L.ref_vectorset_renormalize.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _D, _D, _D]
        L.ref_vectorset_renormalize.restype = C.c_int
        L.ref_order_parameters.argtypes = [_D, C.c_int, C.c_double, _D]
        L.ref_order_parameters.restype = C.c_int
        L.ref_write_records.argtypes = [C.c_int, C.c_int, _D, _D, _D, C.c_char_p, C.c_long]
        L.ref_write_records.restype = C.c_long
        _ref = L
    return _ref


def _d(a):
    return a.ctypes.data_as(_D)


def _f(a):
    return a.ctypes.data_as(_F)


def _i(a):
    return a.ctypes.data_as(_I)


def _u64(a):
    return a.ctypes.data_as(_U64)


class State64:
    """FP64 state in particle-id order: wrapped r, r_original, theta."""

    def __init__(self, x, y, th, xu=None, yu=None):
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.th = np.ascontiguousarray(th, dtype=np.float64)
        self.xu = np.ascontiguousarray(self.x if xu is None else xu, dtype=np.float64).copy()
        self.yu = np.ascontiguousarray(self.y if yu is None else yu, dtype=np.float64).copy()

    def copy(self):
        return State64(self.x.copy(), self.y.copy(), self.th.copy(), self.xu.copy(), self.yu.copy())


def run64(p, state: State64, nsteps, step0=0, fn="orc"):
    """Advance an FP64 state in place with the restatement (fn='orc') or the
    reference's own particle.h (fn='ref')."""
    s = state
    lib = orc().orc64_run if fn == "orc" else ref().ref_run
    rc = lib(C.byref(p), int(nsteps), int(step0), _d(s.x), _d(s.y), _d(s.th), _d(s.xu), _d(s.yu))
    if rc != 0:
        raise RuntimeError(f"{fn} run failed with status {rc}")
    return s


class State32:
    def __init__(self, x, y, th, ix=None, iy=None):
        self.x = np.ascontiguousarray(x, dtype=np.float32).copy()
        self.y = np.ascontiguousarray(y, dtype=np.float32).copy()
        self.th = np.ascontiguousarray(th, dtype=np.float32).copy()
        n = len(self.x)
        self.ix = np.zeros(n, np.int32) if ix is None else np.ascontiguousarray(ix, np.int32).copy()
        self.iy = np.zeros(n, np.int32) if iy is None else np.ascontiguousarray(iy, np.int32).copy()


def run32(p, state: State32, nsteps, step0=0):
    s = state
    rc = orc().orc32_run(C.byref(p), int(nsteps), int(step0), _f(s.x), _f(s.y), _f(s.th),
                         _i(s.ix), _i(s.iy))
    if rc != 0:
        raise RuntimeError(f"mirror run failed with status {rc}")
    return s


def cutoff_events(p, state, nsteps, window, step0=0, cap=1 << 20):
    """Advance `state` (State64: the FP64 restatement, State32: the FP32
    mirror) by nsteps and return the pair evaluations that came within
    `window` of the alignment radius: a structured array of (stage, i, j,
    inside, d), stage counting the force evaluations of this call, i < j,
    inside the run's own predicate and d the run's own distance."""
    fp64 = isinstance(state, State64)
    L = orc()
    start = state.copy() if fp64 else State32(state.x, state.y, state.th, state.ix, state.iy)
    while True:
        st = np.empty(cap, np.int32)
        pi = np.empty(cap, np.int32)
        pj = np.empty(cap, np.int32)
        ins = np.empty(cap, np.int8)
        dist = np.empty(cap, np.float64)
        watch = L.orc64_watch if fp64 else L.orc32_watch
        watch(_i(st), _i(pi), _i(pj), ins.ctypes.data_as(C.POINTER(C.c_int8)), _d(dist), cap,
              float(p.r_align), float(window))
        try:
            (run64 if fp64 else run32)(p, state, nsteps, step0=step0)
            cnt = (L.orc64_watch_count if fp64 else L.orc32_watch_count)()
        finally:
            watch(None, None, None, None, None, 0, 0.0, 0.0)
        if cnt <= cap:
            break
        cap = int(cnt)
        for a in ("x", "y", "th") + (("xu", "yu") if fp64 else ("ix", "iy")):
            setattr(state, a, getattr(start, a).copy())
    ev = np.zeros(cnt, dtype=[("stage", np.int32), ("i", np.int32), ("j", np.int32), ("inside", np.int8),
                              ("d", np.float64)])
    ev["stage"], ev["i"], ev["j"], ev["inside"], ev["d"] = st[:cnt], pi[:cnt], pj[:cnt], ins[:cnt], dist[:cnt]
    return ev


def predicate_mismatches(ev32, ev64, r, window):
    """Pairs (stage, i, j) on which the FP32 and FP64 runs took different sides
    of the alignment cutoff r.  Both runs record every evaluation within
    `window` of r.  A pair recorded by one run only lay within the window
    there and outside it in the other run; it is counted as a mismatch when
    its recorded distance is within window/2 of r (the two runs then differ
    there by more than window/2, and the other run's side is unknown).
    Returns a structured array like cutoff_events'."""
    def key(e):
        return ((e["stage"].astype(np.int64) << 42) | (e["i"].astype(np.int64) << 21)
                | e["j"].astype(np.int64))
    k32, k64 = key(ev32), key(ev64)
    _, a, b = np.intersect1d(k32, k64, return_indices=True)
    out = [ev32[a][ev32[a]["inside"] != ev64[b]["inside"]]]
    for e, k, other in ((ev32, k32, k64), (ev64, k64, k32)):
        lone = e[~np.isin(k, other)]
        out.append(lone[np.abs(lone["d"] - r) < 0.5 * window])
    return np.concatenate(out)


def stages_per_step(p):
    return {1: 1, 2: 2, 4: 4}[int(p.integrator)] if p.model in (3, 4, 5) else 1


def cutoff_divergence(p, x, y, th, nsteps, window=1e-3, step0=0, hops=1, close=0.0):
    """The FP64 restatement and the FP32 mirror (the kernels' arithmetic) run
    side by side from the same state for nsteps, step by step, recording the
    pair evaluations near the hard alignment cutoff.  Where the two
    precisions put a pair on different sides of the cutoff, the torques of
    its two particles jump (by ~ dt g / n_i) and their headings part by far
    more than rounding; their neighbours then feel the changed headings
    through their own alignment sums.  Returns (final State64, final
    State32, the mismatched pair evaluations, level): level 0 for members of
    a mismatched pair (from that step on), level h <= hops for particles
    within the alignment radius of a level h-1 particle at any later step,
    99 for the rest.  With close > 0, particles closer than `close` to
    another at the start of a step are level 0 as well: the continuous
    model's alpha torque alpha (dr x v)/(pi d) takes its direction from dr/d,
    whose FP32 rounding error grows as 1/d where two particles (which do not
    repel) pass through each other."""
    s64, s32 = State64(x, y, th), State32(x, y, th)
    nst = stages_per_step(p)
    level = np.full(p.n, 99, np.int32)
    found = []

    def hop():
        if not (level < hops).any():
            return
        pr = pairs64(s64.x, s64.y, p.L, p.r_align)
        a = (pr >> 32).astype(np.int64)
        b = (pr & 0xFFFFFFFF).astype(np.int64)
        la, lb = level[a].copy(), level[b].copy()
        np.minimum.at(level, b, np.where(la < hops, la + 1, 99))
        np.minimum.at(level, a, np.where(lb < hops, lb + 1, 99))

    for t in range(nsteps):
        if close > 0:
            pr = pairs64(s64.x, s64.y, p.L, close)
            level[(pr >> 32).astype(np.int64)] = 0
            level[(pr & 0xFFFFFFFF).astype(np.int64)] = 0
        hop()
        e64 = cutoff_events(p, s64, 1, window, step0=step0 + t)
        e32 = cutoff_events(p, s32, 1, window, step0=step0 + t)
        mm = predicate_mismatches(e32, e64, p.r_align, window)
        mm["stage"] += t * nst
        level[mm["i"]] = 0
        level[mm["j"]] = 0
        found.append(mm)
    hop()
    return s64, s32, np.concatenate(found), level


def pairs64(x, y, L, r, cap=None):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    n = len(x)
    cap = cap or max(16, 8 * n)
    pi = np.empty(cap, np.int32)
    pj = np.empty(cap, np.int32)
    cnt = orc().orc64_pairs(n, _d(x), _d(y), float(L), float(r), _i(pi), _i(pj), cap)
    if cnt > cap:
        return pairs64(x, y, L, r, cap=int(cnt))
    return _sorted_pairs(pi[:cnt], pj[:cnt])


def tumble_steps(p):
    """Length in steps of a run-and-tumble tumble, as the kernels count it."""
    q = p.copy()
    q.model = abi.MODEL_BEADS
    q.rot_noise = abi.NOISE_TUMBLE
    return int(orc().orc32_tumble_steps(C.byref(q)))


def radial32(x, y, L, r_max, nbins, closed=False):
    """Ordered-pair radial histogram, FP32 as spp_radial_distribution computes it (O(N^2));
    closed: a closed box (plain differences)."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros(nbins, np.uint64)
    orc().orc32_radial(_f(x), _f(y), len(x), float(L), float(r_max), int(nbins), _u64(out), int(bool(closed)))
    return out


def pair_distribution32(x, y, c, s, lx, ly, gx, gy):
    """Body-frame histogram [gx][gy], FP32 as spp_pair_distribution computes it (O(N^2))."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (x, y, c, s)]
    out = np.zeros(gx * gy, np.uint64)
    orc().orc32_pair_distribution(*[_f(a) for a in arrs], len(arrs[0]), float(lx), float(ly), int(gx),
                                  int(gy), _u64(out))
    return out.reshape(gx, gy)


def pairs32(p, x, y, r, cap=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    n = len(x)
    q = p.replace(n=n)
    cap = cap or max(16, 8 * n)
    pi = np.empty(cap, np.int32)
    pj = np.empty(cap, np.int32)
    cnt = orc().orc32_pairs(C.byref(q), _f(x), _f(y), float(r), _i(pi), _i(pj), cap)
    if cnt > cap:
        return pairs32(p, x, y, r, cap=int(cnt))
    return _sorted_pairs(pi[:cnt], pj[:cnt])


def _sorted_pairs(pi, pj):
    a = np.minimum(pi, pj).astype(np.int64)
    b = np.maximum(pi, pj).astype(np.int64)
    key = np.sort(a * (1 << 32) + b)
    return key


def cells64(x, y, L, D, rule):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    cx = np.empty(len(x), np.int32)
    cy = np.empty(len(x), np.int32)
    orc().orc_cells(len(x), _d(x), _d(y), float(L), int(D), int(rule), _i(cx), _i(cy))
    return cx, cy


def cells32(p, x, y, D, rule):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    q = p.replace(n=len(x))
    cx = np.empty(len(x), np.int32)
    cy = np.empty(len(x), np.int32)
    orc().orc32_cells(C.byref(q), _f(x), _f(y), int(D), int(rule), _i(cx), _i(cy))
    return cx, cy


def polarization(th):
    th = np.ascontiguousarray(th, np.float64)
    px = C.c_double()
    py = C.c_double()
    P = orc().orc_polarization(len(th), _d(th), C.byref(px), C.byref(py))
    return P, px.value, py.value


def philox(ctr, key, round_keys=False):
    """Philox4x32-10 of counter ctr and key (k0, k1); round_keys=True takes
    the kernels' route through precomputed round keys."""
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    (orc().orc32_philox_ks if round_keys else orc().orc32_philox)(c, k, o)
    return tuple(o)


def fx_sum(x):
    x = np.ascontiguousarray(x, np.float32)
    hi, lo, v = C.c_int32(), C.c_int32(), C.c_float()
    orc().orc32_fx_sum(len(x), _f(x), C.byref(hi), C.byref(lo), C.byref(v))
    return hi.value, lo.value, v.value


def rsqrt32(x):
    return float(orc().orc32_rsqrt(float(x)))


def lyap_init32(p, K, seed):
    V = np.empty(K * 3 * p.n, np.float32)
    rc = orc().orc32_lyap_init(C.byref(p), int(K), int(seed), _f(V))
    if rc:
        raise RuntimeError(f"mirror lyap init failed {rc}")
    return V


def lyap_run32(p, state: State32, V, nsteps, renorm_every, step0=0):
    """Mirror of the kernels' base + tangent steps; V ([K*3*n] float32) and
    the returned log-stretch sums are updated in place."""
    K = V.size // (3 * p.n)
    ls = np.zeros(K, np.float64)
    s = state
    rc = orc().orc32_lyap_run(C.byref(p), int(nsteps), int(step0), int(renorm_every), K, _f(s.x),
                              _f(s.y), _f(s.th), _i(s.ix), _i(s.iy), _f(V), _d(ls))
    if rc:
        raise RuntimeError(f"mirror lyap run failed {rc}")
    return ls


def lyap_tangent64(p, state: State64, V, nsteps, renorm_every):
    K = V.size // (3 * p.n)
    ls = np.zeros(K, np.float64)
    s = state
    rc = orc().orc64_lyap_tangent(C.byref(p), int(nsteps), int(renorm_every), K, _d(s.x), _d(s.y),
                                  _d(s.th), _d(s.xu), _d(s.yu), _d(V), _d(ls))
    if rc:
        raise RuntimeError(f"oracle lyap tangent failed {rc}")
    return ls


def lyap_clone64(p, state: State64, V, n_intervals, tau, eps=1e-7):
    K = V.size // (3 * p.n)
    ls = np.zeros(K, np.float64)
    s = state
    rc = orc().orc64_lyap_clone(C.byref(p), int(n_intervals), int(tau), K, float(eps), _d(s.x),
                                _d(s.y), _d(s.th), _d(s.xu), _d(s.yu), _d(V), _d(ls))
    if rc:
        raise RuntimeError(f"oracle lyap clone failed {rc}")
    return ls


def gram_schmidt64(V, n, eps, fn="oracle", L=32.0):
    """Orthonormalises K deviation vectors [K][3][n] (a copy) and returns
    (U, log growth ratios log(R_aa / eps)): the oracle's modified
    Gram-Schmidt, or with fn="ref" the reference's own VectorSet::
    Renormalize(us) and LyapunovBox growth ratio (oracle/ref_harness.cpp)."""
    V = np.ascontiguousarray(V, np.float64).copy()
    K = V.size // (3 * n)
    if fn == "ref":
        U = np.empty_like(V)
        ratio = np.empty(K, np.float64)
        rc = ref().ref_vectorset_renormalize(K, n, float(L), float(eps), _d(V), _d(U), _d(ratio))
        if rc:
            raise RuntimeError(f"reference renormalisation failed {rc}")
        return U, np.log(ratio)
    ls = np.zeros(K, np.float64)
    rc = orc().orc64_gram_schmidt(K, n, _d(V), _d(ls), float(eps))
    if rc:
        raise RuntimeError(f"oracle Gram-Schmidt failed {rc}")
    return V, ls


MATH_FNS = {"sin": 0, "cos": 1, "atan2": 2, "log": 3, "exp": 4, "wrap": 5}


def math32(fn, a, b=None):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(a if b is None else b, np.float32)
    out = np.empty_like(a)
    orc().orc32_math(MATH_FNS[fn], len(a), _f(a), _f(b), _f(out))
    return out


def circle_torque32(p, x, y, th):
    """The kernels' FP32 circle torque (spp_circle_torque) of one particle."""
    return float(orc().orc32_circle_torque(C.byref(p), float(x), float(y), float(th)))


def wall_terms(p, x, y, th, fn="orc64"):
    """Walls of p's closed box on one particle: {fx, fy, RepulsiveParticle
    torque, ContinuousParticle torque} from the FP64 restatement
    (fn='orc64'), the reference's own Wall::Interact (fn='ref'), or the
    kernels' FP32 arithmetic (fn='orc32': {fx, fy, torque})."""
    if fn == "orc32":
        out = np.zeros(3, np.float32)
        orc().orc32_wall_terms(C.byref(p), float(x), float(y), float(th), _f(out))
        return out
    out = np.zeros(4, np.float64)
    lib = orc().orc64_wall_terms if fn == "orc64" else ref().ref_wall_terms
    lib(C.byref(p), float(x), float(y), float(th), _d(out))
    return out

