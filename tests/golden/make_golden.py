"""Regenerate tests/golden/reference_runs.npz from the reference's own code.

Runs the reference's particle classes (shared/particle.h, compiled by
oracle/build.py from the reference checkout into oracle/_ref/libspp_ref.so,
with the GSL calls answered by the Philox shim) on small seeded cases and
stores inputs and outputs.  The fixtures pin the FP64 restatement
(oracle/spp_oracle64.c) where the reference checkout is absent.

    python tests/golden/make_golden.py [runs] [gram_schmidt] [order_parameters] [records]
    (default: all four)

reference_gram_schmidt.npz pins the Lyapunov clone method's
renormalisation (shared/vector-set.h:118-127, parallel/lyapunovbox.h:
177-181) the same way, and reference_order_parameters.npz the analysis
statistics (analyze/statistics.h:35-82, analyze/analyze.h:121-146), and
reference_records.npz the particle records of the .bin frame writer
(shared/particle.h:759-764, 1022-1045).
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from spp_gb300 import abi, configs  # noqa: E402
from oracle import oracle as O  # noqa: E402


def lattice(n_side, spacing, L):
    g = (np.arange(n_side) * spacing - L + 0.25 * spacing).astype(np.float64)
    X, Y = np.meshgrid(g, g)
    return X.ravel(), Y.ravel()


def rtp_case(integ):
    """RTPChain (run and tumble) swimmers inside rings: tumbles start often
    (rate 20, dt 0.002) and last 0.03 (15 steps)."""
    p = configs.vesicle_config(n_rings=4, ring_size=40, swimmers_per_ring=8, L=20.0,
                               integrator=integ, seed=9)
    x, y, th = configs.vesicle_state(p)
    p.sigma_rep, p.r_rep, p.k_rep = 0.5, 0.55, 1.0
    p.bond_rest, p.k_bond, p.kappa_bend = 0.55, 30.0, 0.0
    p.dt = 0.002
    p.rot_noise = abi.NOISE_TUMBLE
    p.tumble_rate, p.tumble_time, p.tumble_torque = 20.0, 0.03, 3.0
    return p, x.astype(np.float64), y.astype(np.float64), th.astype(np.float64)


def chain_case(integ):
    """Free chiral trimers (ActiveBrownianChain, nb = 3) packed closely
    enough to collide."""
    p = configs.chain_config(n=144, chain_beads=3, integrator=integ, seed=5, spacing=1.7)
    p.torque0 = 0.3
    x, y, th = configs.chain_state(p)
    return p, x.astype(np.float64), y.astype(np.float64), th.astype(np.float64)


def dimer_case(integ):
    """Dimer swimmers (nb = 2) inside ring membranes."""
    p = configs.vesicle_config(n_rings=4, ring_size=40, swimmers_per_ring=8, L=20.0,
                               integrator=integ, seed=9)
    x, y, th = configs.vesicle_state(p)
    p.sigma_rep, p.r_rep, p.k_rep = 0.5, 0.55, 1.0
    p.bond_rest, p.k_bond, p.kappa_bend = 0.55, 30.0, 0.0
    p.Dr, p.dt = 0.2, 0.002
    p.chain_beads, p.bead_separation, p.sigma_chain, p.r_chain = 2, 0.5, 0.5, 0.55
    return p, x.astype(np.float64), y.astype(np.float64), th.astype(np.float64)


def cases():
    out = []
    for integ, name in ((abi.INT_EULER, "euler"), (abi.INT_RK2, "rk2"), (abi.INT_RK4, "rk4")):
        p = configs.reference_defaults(abi.MODEL_ABP)
        p.n, p.L, p.Dr, p.dt, p.seed, p.integrator = 400, 10.0, 0.1, 0.005, 5, integ
        x, y = lattice(20, 1.0, p.L)
        _, _, th = configs.random_state(p.n, p.L, seed=7)
        out.append((f"repulsive_{name}", p, x, y, th.astype(np.float64), 50))
    for model, name in ((abi.MODEL_VICSEK_REF_ANGLE, "vicsek_angle"),
                        (abi.MODEL_VICSEK_REF_VECTOR, "vicsek_vector")):
        p = configs.vicsek_config(n=1024, L=16.0, model=model, seed=0)
        x, y, th = configs.random_state(p.n, p.L, seed=3)
        out.append((name, p, x.astype(np.float64), y.astype(np.float64), th.astype(np.float64), 20))
    for integ, name in ((abi.INT_EULER, "beads_euler"), (abi.INT_RK2, "beads_rk2")):
        # ActiveBrownianChain (nb = 1) rings + swimmers with the reference's
        # membrane repulsion (sigma 0.5, cutoff 0.55) and Spring bonds
        p = configs.vesicle_config(n_rings=4, ring_size=40, swimmers_per_ring=8, L=20.0,
                                   integrator=integ)
        x, y, th = configs.vesicle_state(p)  # rings of unit bonds, then stretched below
        p.sigma_rep, p.r_rep, p.k_rep = 0.5, 0.55, 1.0
        p.bond_rest, p.k_bond, p.kappa_bend = 0.55, 30.0, 0.0
        p.Dr, p.dt = 0.2, 0.002
        out.append((name, p, x.astype(np.float64), y.astype(np.float64), th.astype(np.float64), 60))
    for integ, name in ((abi.INT_EULER, "rtp_euler"), (abi.INT_RK2, "rtp_rk2")):
        out.append((name, *rtp_case(integ), 80))
    for integ, name in ((abi.INT_EULER, "chains_euler"), (abi.INT_RK2, "chains_rk2")):
        out.append((name, *chain_case(integ), 150))
    out.append(("dimers_rk2", *dimer_case(abi.INT_RK2), 100))
    p = configs.reference_defaults(abi.MODEL_CONTINUOUS)
    p.n, p.L, p.Dr, p.dt, p.v0, p.seed = 1024, 16.0, 0.05, 0.01, 0.5, 11
    x, y, th = configs.random_state(p.n, p.L, seed=3)
    out.append(("continuous_euler", p, x.astype(np.float64), y.astype(np.float64),
                th.astype(np.float64), 20))
    return out


WALL_SEGMENTS = [[-5.0, -3.0, 4.0, 6.0], [2.0, -8.0, -6.0, 1.0], [-20.0, -20.0, -20.0, 20.0],
                 [20.0, 20.0, 20.0, -20.0]]


def wall_case(model):
    """Wall::Interact of the reference on single particles near four
    segments (two oblique, two box walls): parameters and sample points."""
    p = configs.reference_defaults(model)
    p.L, p.n = 20.0, 1
    p.boundary = abi.BOUNDARY_WALLS
    p.n_walls = 4
    abi.set_field(p, "walls", WALL_SEGMENTS)
    p.A_w, p.sigma_w, p.r_c_w, p.r_f_w, p.g_w, p.g_w_cont = 3.0, 0.4, 1.5, 1.2, 2.0, 20.0
    rng = np.random.default_rng(11)
    pts = []
    for t in range(400):
        w = WALL_SEGMENTS[t % 4]
        u = rng.uniform(-0.2, 1.2)
        pts.append((w[0] + u * (w[2] - w[0]) + rng.uniform(-1.6, 1.6),
                    w[1] + u * (w[3] - w[1]) + rng.uniform(-1.6, 1.6), rng.uniform(-np.pi, np.pi)))
    return p, np.array(pts, np.float64)


def gram_schmidt_cases():
    """Deviation vectors [K][3][n] at the clone method's scale (eps = 1e-7):
    independent ones, and a set whose later vectors are the earlier ones
    plus 1e-3 of new noise (nearly dependent, where modified and classical
    Gram-Schmidt part)."""
    n, K, eps = 300, 5, 1e-7
    rng = np.random.default_rng(21)
    free = rng.standard_normal((K, 3 * n)) * eps
    close = np.empty((K, 3 * n))
    close[0] = rng.standard_normal(3 * n) * eps
    for a in range(1, K):
        close[a] = close[a - 1] + 1e-3 * rng.standard_normal(3 * n) * eps
    return n, eps, {"independent": free.ravel(), "nearly_dependent": close.ravel()}


def gram_schmidt_fixture():
    """tests/golden/reference_gram_schmidt.npz: the reference's
    VectorSet::Renormalize(us) and LyapunovBox growth ratios."""
    n, eps, cases_ = gram_schmidt_cases()
    blob = {"n": np.array(n), "eps": np.array(eps)}
    for name, V in cases_.items():
        U, logr = O.gram_schmidt64(V, n, eps, fn="ref")
        blob[f"{name}/in"], blob[f"{name}/U"], blob[f"{name}/log_ratio"] = V, U, logr
    path = Path(__file__).resolve().parent / "reference_gram_schmidt.npz"
    np.savez_compressed(path, **blob)
    print(path, path.stat().st_size, "bytes")


ORDER_KEYS = ["mean", "mean_square", "variance", "std", "min", "max", "corr_len", "error", "sigma2",
              "p4_mean", "binder_reference"]


def ar1_series(T, phi, seed, mean=0.6, sd=0.05):
    """A polarization-like AR(1) series: correlation time ~ 1 / (1 - phi)."""
    rng = np.random.default_rng(seed)
    x = np.empty(T)
    x[0] = mean
    for t in range(1, T):
        x[t] = mean + phi * (x[t - 1] - mean) + sd * rng.standard_normal()
    return x


ORDER_CASES = [(600, 0.9, 1), (1000, 0.0, 2), (257, 0.98, 3), (2, 0.5, 4), (5000, 0.995, 5)]


def order_parameters_fixture():
    """tests/golden/reference_order_parameters.npz: the reference's own
    Stat::Compute / Find_Correlation_Length and the combination of
    Compute_Order_Parameters on AR(1) series (area 4096)."""
    import ctypes as C
    blob = {"keys": np.frombuffer(json.dumps(ORDER_KEYS).encode(), dtype=np.uint8)}
    for T, phi, seed in ORDER_CASES:
        x = ar1_series(T, phi, seed)
        out = np.zeros(len(ORDER_KEYS))
        rc = O.ref().ref_order_parameters(x.ctypes.data_as(C.POINTER(C.c_double)), T, 4096.0,
                                          out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc:
            raise SystemExit(f"reference statistics failed on case {T}")
        blob[f"T{T}_seed{seed}/in"], blob[f"T{T}_seed{seed}/out"] = x, out
    path = Path(__file__).resolve().parent / "reference_order_parameters.npz"
    np.savez_compressed(path, **blob)
    print(path, path.stat().st_size, "bytes")


def records_fixture():
    """tests/golden/reference_records.npz: the bytes of the reference's own
    particle Write methods (RepulsiveParticle, ActiveBrownianChain membrane
    bead and swimmer) for seeded unwrapped positions and headings."""
    import ctypes as C
    rng = np.random.default_rng(31)
    n = 200
    xu = rng.uniform(-5e4, 5e4, n)
    yu = rng.uniform(-5e4, 5e4, n)
    th = rng.uniform(-np.pi, np.pi, n)
    blob = {"xu": xu, "yu": yu, "theta": th}
    for kind in (0, 1, 2):
        buf = C.create_string_buffer(16 * n)
        m = O.ref().ref_write_records(kind, n, O._d(xu), O._d(yu), O._d(th), buf, 16 * n)
        blob[f"kind{kind}"] = np.frombuffer(buf.raw[:m], dtype=np.uint8)
    path = Path(__file__).resolve().parent / "reference_records.npz"
    np.savez_compressed(path, **blob)
    print(path, path.stat().st_size, "bytes")


def main(parts=("runs", "gram_schmidt", "order_parameters", "records")):
    if O.ref() is None:
        raise SystemExit("reference checkout not found: cannot regenerate the fixtures")
    if "records" in parts:
        records_fixture()
    if "gram_schmidt" in parts:
        gram_schmidt_fixture()
    if "order_parameters" in parts:
        order_parameters_fixture()
    if "runs" not in parts:
        return
    blob = {}
    meta = {}
    for name, p, x, y, th, steps in cases():
        s = O.State64(x, y, th)
        blob[f"{name}/in"] = np.stack([s.x, s.y, s.th, s.xu, s.yu])
        O.run64(p, s, steps, fn="ref")
        blob[f"{name}/out"] = np.stack([s.x, s.y, s.th, s.xu, s.yu])
        meta[name] = {"params": {k: v for k, v in p.as_dict().items()}, "steps": steps}
    for model, name in ((abi.MODEL_ABP, "walls_abp"), (abi.MODEL_CONTINUOUS, "walls_continuous"),
                        (abi.MODEL_VICSEK_REF_ANGLE, "walls_vicsek")):
        p, pts = wall_case(model)
        blob[f"{name}/in"] = pts
        blob[f"{name}/out"] = np.array([O.wall_terms(p, *q, fn="ref") for q in pts])
        meta[name] = {"params": {k: v for k, v in p.as_dict().items()}, "steps": 0}
    blob["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = Path(__file__).resolve().parent / "reference_runs.npz"
    np.savez_compressed(path, **blob)
    print(path, path.stat().st_size, "bytes")


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or ("runs", "gram_schmidt", "order_parameters", "records"))
