"""Parameter presets and initial conditions.

Presets:
  * ``reference_defaults(model)``: the reference's static initialisers
    (shared/particle.h:138-140, 249-250, 373-378, 774-786, 1049-1056).
  * ``vicsek_config(...)``: discrete Vicsek, N=4096, 64x64 box (L=32),
    v0=0.5, r=1, eta=0.3, dt=1 (the CPU-runnable FP64 workload).
  * ``abp_config(...)``: repulsive active Brownian / Vicsek, N=1,048,576,
    1024x1024 box (L=512), harmonic k(1 - r/2a) with a=0.5, k=10,
    (g/n_i) sum sin alignment within r=1, D_r=0.1, v0=1, RK2 dt=0.005,
    Verlet skin 0.3 (the headline GPU workload).

Initial conditions are drawn from the same Philox4x32-10 stream the kernels
use (stream tags SPP_RNG_INIT_POS / SPP_RNG_INIT_ANGLE), so they are
identical on every machine; this numpy version is checked against the C
implementation in the tests.
"""
import math

import numpy as np

from . import abi

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
RNG_ROT_NOISE, RNG_VICSEK, RNG_INIT_POS, RNG_INIT_ANGLE = 1, 2, 3, 4


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 (Salmon et al., SC'11) on uint32 arrays."""
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint32).copy() for v in (c0, c1, c2, c3))
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    mask = np.uint64(0xFFFFFFFF)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = M0 * c0.astype(np.uint64)
            p1 = M1 * c2.astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & mask).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & mask).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0 = np.uint32(k0 + W0)
            k1 = np.uint32(k1 + W1)
    return c0, c1, c2, c3


def draw(seed, system, pids, step, stream):
    pids = np.asarray(pids, dtype=np.uint32)
    z = np.zeros_like(pids)
    return philox4x32_10(pids, z + np.uint32(step), z + np.uint32(stream), z + np.uint32(system),
                         seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)


def u01_f32(bits):
    return (bits >> np.uint32(8)).astype(np.float32) * np.float32(5.9604644775390625e-08)


def random_state(n, L, seed, system=0):
    """Uniform positions in [-L, L)^2 and headings in [-pi, pi), float32,
    from the Philox init streams (Random_Formation, shared/set-up.h:153-163,
    with the GSL draws replaced)."""
    ids = np.arange(n, dtype=np.uint32)
    a = draw(seed, system, ids, 0, RNG_INIT_POS)
    b = draw(seed, system, ids, 0, RNG_INIT_ANGLE)
    Lf = np.float32(L)
    x = (np.float32(2.0) * u01_f32(a[0]) - np.float32(1.0)) * Lf
    y = (np.float32(2.0) * u01_f32(a[1]) - np.float32(1.0)) * Lf
    th = (np.float32(2.0) * u01_f32(b[0]) - np.float32(1.0)) * np.float32(math.pi)
    # (2u-1)*L rounds up to L for u near 1 when L is not a power of two; keep [-L, L)
    x = np.where(x >= Lf, -Lf, x).astype(np.float32)
    y = np.where(y >= Lf, -Lf, y).astype(np.float32)
    return x.astype(np.float32), y.astype(np.float32), th.astype(np.float32)


def reference_defaults(model) -> abi.SppParams:
    """The reference's static initialisers for a model."""
    p = abi.new_params(model=model, n=0, seed=10, L=64.0, dt=1.0 / 1024, v0=1.0, Dr=0.0, eta=0.0,
                       g=1.0, alpha=0.0, r_align=1.0, r_rep=0.0, k_rep=0.0, sigma_rep=1.0,
                       skin=0.0, beta_push=2.5, r_push=0.127, mu=0.5, k_perp=1.0, torque0=0.0,
                       k_bond=0.0, bond_rest=1.0, kappa_bend=0.0, integrator=abi.INT_EULER,
                       force_law=abi.FORCE_NONE, align_mode=abi.ALIGN_REFERENCE)
    if model == abi.MODEL_ABP:  # RepulsiveParticle, shared/particle.h:774-786
        p.integrator = abi.INT_RK2
        p.force_law = abi.FORCE_R12_TRUNC
        p.k_rep, p.sigma_rep, p.r_align, p.r_rep, p.g = 2.0, 1.0, 1.1, 1.2, 1.0
    elif model == abi.MODEL_CONTINUOUS:  # ContinuousParticle, :373-378
        p.g, p.alpha = 4.0, 0.5
    elif model == abi.MODEL_BEADS:  # ActiveBrownianChain, :1049-1056
        p.force_law = abi.FORCE_R12_TRUNC
        p.k_rep, p.sigma_rep, p.r_rep = 1.0, 0.5, 0.55
        p.mu, p.k_perp = 0.5, 1.0
        p.integrator = abi.INT_RK2
    return p


def vicsek_config(n=4096, L=32.0, eta=0.3, seed=0, model=abi.MODEL_VICSEK) -> abi.SppParams:
    """Plain Vicsek: N=4096 in a 64x64 periodic box, v0=0.5, r=1, eta=0.3, dt=1."""
    p = reference_defaults(model)
    p.n, p.L, p.eta, p.seed = n, L, eta, seed
    p.v0, p.r_align, p.dt = 0.5, 1.0, 1.0
    p.integrator = abi.INT_EULER
    p.skin = 0.0
    return p


def abp_config(n=1 << 20, L=512.0, seed=1, integrator=abi.INT_RK2) -> abi.SppParams:
    """Repulsive ABP / Vicsek: N=1,048,576 disks (a=0.5) in a 1024x1024 box."""
    p = reference_defaults(abi.MODEL_ABP)
    p.n, p.L, p.seed = n, L, seed
    p.integrator = integrator
    p.force_law = abi.FORCE_HARMONIC
    p.align_mode = abi.ALIGN_MEAN
    p.k_rep, p.r_rep = 10.0, 1.0          # k (1 - r / 2a), 2a = 1
    p.g, p.r_align = 1.0, 1.0
    p.Dr, p.v0, p.dt = 0.1, 1.0, 0.005
    p.skin = 0.3
    return p


WCA_CUTOFF = 2.0 ** (1.0 / 6.0)


def vesicle_config(n_rings=1024, ring_size=128, swimmers_per_ring=32, L=None, seed=2,
                   integrator=abi.INT_RK4) -> abi.SppParams:
    """Ring vesicles with swimmers: n_rings rings of ring_size beads (radius
    0.5, bonds k = 100 at rest length 1, bending kappa = 10), each enclosing
    swimmers_per_ring active Brownian swimmers (v0 = 1, D_r = 0.05); a
    WCA-like truncated r^-12 repulsion (R12_Repulsive_Truncated with
    sigma = 1, cutoff 2^(1/6)) acts between all bodies; RK4, dt = 0.002.

    The box is sized to 30% area fraction counting each vesicle's enclosed
    disk of radius R + a, R = 0.5 / sin(pi / M) (set-up.h:299): 1024 rings
    of 128 beads give a side of 2162 (L = 1081).  Counting bead disks alone
    would give a box smaller than the rings themselves."""
    R = 0.5 / math.sin(math.pi / ring_size)
    if L is None:
        area = n_rings * math.pi * (R + 0.5) ** 2 / 0.30
        L = 0.5 * math.sqrt(area)
    p = reference_defaults(abi.MODEL_BEADS)
    p.n_rings, p.ring_size = n_rings, ring_size
    p.n = n_rings * ring_size + n_rings * swimmers_per_ring
    p.L, p.seed, p.integrator = float(L), seed, integrator
    p.force_law = abi.FORCE_R12_TRUNC
    p.sigma_rep, p.r_rep, p.k_rep = 1.0, WCA_CUTOFF, 1.0
    p.k_bond, p.bond_rest, p.kappa_bend = 100.0, 1.0, 10.0
    p.mu, p.k_perp, p.torque0 = 0.5, 1.0, 0.0
    p.v0, p.Dr, p.dt, p.skin = 1.0, 0.05, 0.002, 0.3
    return p


def vesicle_state(p, swimmers_per_ring=None, seed=None):
    """Rings on a jittered square grid (centres), beads evenly on each ring
    (Ring_Membrane, shared/set-up.h:292-316), swimmers on a small square
    lattice (spacing 1.5) around each centre with random headings."""
    seed = p.seed if seed is None else seed
    M, nr = p.ring_size, p.n_rings
    ns = (p.n - nr * M) // max(nr, 1) if swimmers_per_ring is None else swimmers_per_ring
    L = p.L
    R = 0.5 * p.bond_rest / math.sin(math.pi / M)
    G = int(math.ceil(math.sqrt(nr)))
    spacing = 2 * L / G
    slack = max(0.0, 0.5 * (spacing - 2 * R - 2.0))
    ids = np.arange(nr, dtype=np.uint32)
    jit = draw(seed, 0, ids, 0, RNG_INIT_POS)
    cx = -L + (np.arange(nr) % G + 0.5) * spacing + (2 * u01_f32(jit[0]).astype(np.float64) - 1) * 0.5 * slack
    cy = -L + (np.arange(nr) // G + 0.5) * spacing + (2 * u01_f32(jit[1]).astype(np.float64) - 1) * 0.5 * slack
    ang = 2 * math.pi * np.arange(M) / M
    bx = (cx[:, None] + R * np.cos(ang)[None, :]).ravel()
    by = (cy[:, None] + R * np.sin(ang)[None, :]).ravel()
    bth = np.zeros(nr * M)
    # swimmer lattice: the ns sites closest to the centre
    g = np.arange(-12, 13) * 1.5
    gx, gy = np.meshgrid(g, g)
    order = np.argsort(gx.ravel() ** 2 + gy.ravel() ** 2 + 1e-6 * gx.ravel(), kind="stable")
    sx0, sy0 = gx.ravel()[order][:ns], gy.ravel()[order][:ns]
    if ns and np.max(np.hypot(sx0, sy0)) > R - 2.0:
        raise ValueError("too many swimmers for the ring size")
    sid = np.arange(nr * ns, dtype=np.uint32)
    sw = draw(seed, 0, sid, 0, RNG_INIT_ANGLE)
    sx = (cx[:, None] + sx0[None, :]).ravel() + 0.2 * (2 * u01_f32(sw[1]).astype(np.float64) - 1)
    sy = (cy[:, None] + sy0[None, :]).ravel() + 0.2 * (2 * u01_f32(sw[2]).astype(np.float64) - 1)
    sth = (2 * u01_f32(sw[0]).astype(np.float64) - 1) * math.pi
    x = np.concatenate([bx, sx])
    y = np.concatenate([by, sy])
    th = np.concatenate([bth, sth])
    # wrap into [-L, L)
    x = x - 2 * L * np.floor((x + L) / (2 * L))
    y = y - 2 * L * np.floor((y + L) / (2 * L))
    x = x.astype(np.float32)
    y = y.astype(np.float32)
    Lf = np.float32(L)
    x = np.where(x >= Lf, -Lf, x).astype(np.float32)
    y = np.where(y >= Lf, -Lf, y).astype(np.float32)
    return x, y, th.astype(np.float32)


def chain_config(n=4096, chain_beads=3, separation=0.5, sigma=0.5, r_chain=0.55, spacing=2.0,
                 seed=4, integrator=abi.INT_RK2) -> abi.SppParams:
    """Free multi-bead swimmers, no membranes: n chains of chain_beads beads
    (ActiveBrownianChain with nb > 1, shared/particle.h:856-1012), beads
    separation apart, R12 between beads (sigma, cutoff r_chain, A = 1), on a
    square lattice of the given spacing (L = spacing sqrt(n) / 2); v0 = 1,
    D_r = 0.1, no intrinsic torque."""
    G = int(math.ceil(math.sqrt(n)))
    p = reference_defaults(abi.MODEL_BEADS)
    p.n_rings, p.ring_size = 0, 0
    p.n, p.seed, p.integrator = n, seed, integrator
    p.L = 0.5 * spacing * G
    p.force_law = abi.FORCE_R12_TRUNC
    p.k_rep = 1.0
    p.chain_beads, p.bead_separation, p.sigma_chain, p.r_chain = chain_beads, separation, sigma, r_chain
    p.v0, p.Dr, p.dt, p.skin, p.torque0 = 1.0, 0.1, 0.002, 0.3, 0.0
    return p


def chain_state(p, seed=None):
    """Chains of a chain_config on their square lattice, random headings:
    with spacing > (nb - 1) separation + r_chain no two chains touch."""
    seed = p.seed if seed is None else seed
    G = int(math.ceil(math.sqrt(p.n)))
    spacing = 2 * p.L / G
    ids = np.arange(p.n, dtype=np.uint32)
    r = draw(seed, 0, ids, 0, RNG_INIT_ANGLE)
    x = (-p.L + (ids % G + 0.5) * spacing).astype(np.float32)
    y = (-p.L + (ids // G + 0.5) * spacing).astype(np.float32)
    th = ((2 * u01_f32(r[0]).astype(np.float64) - 1) * math.pi).astype(np.float32)
    return x, y, th


def walls_config(n=4096, L=40.0, model=abi.MODEL_ABP, integrator=abi.INT_RK2, seed=6,
                 extra_walls=((-10.0, -4.0, 8.0, 12.0), (6.0, -14.0, -12.0, 2.0))):
    """A closed box (the reference built without PERIODIC_BOUNDARY_CONDITION):
    the four box walls plus extra segments, with the wall interactions of
    RepulsiveParticle (screened repulsion A_w = 3, sigma_w = 0.4, cutoff 1.5;
    alignment g_w = 2 within 1.2) or ContinuousParticle (gw = 20).  ABP: the
    reference's R12 pair law and alignment; continuous: g = 1, alpha = 0."""
    p = reference_defaults(model)
    p.n, p.L, p.seed, p.integrator = n, L, seed, integrator
    p.boundary = abi.BOUNDARY_WALLS
    p.n_walls = len(extra_walls)
    abi.set_field(p, "walls", [list(w) for w in extra_walls])
    p.A_w, p.sigma_w, p.r_c_w, p.r_f_w, p.g_w, p.g_w_cont = 3.0, 0.4, 1.5, 1.2, 2.0, 20.0
    p.Dr, p.dt, p.skin = 0.1, 0.005, 0.3
    if model == abi.MODEL_CONTINUOUS:
        p.g, p.alpha, p.v0, p.dt = 1.0, 0.0, 0.5, 0.01
    if model in (abi.MODEL_VICSEK_REF_ANGLE, abi.MODEL_VICSEK_REF_VECTOR):
        p.v0, p.r_align, p.dt, p.eta = 0.5, 1.0, 1.0, 0.3
    return p


def vicsek_walls_state(p, seed=None, half=None):
    """Discrete Vicsek particles of a closed box: uniform in the central
    square of half-width `half` (default L/2, so that they stay inside the
    box for a few dozen steps: VicsekParticle feels walls only as alignment,
    nothing keeps it in), headings uniform."""
    seed = p.seed if seed is None else seed
    half = p.L / 2 if half is None else half
    ids = np.arange(p.n, dtype=np.uint32)
    r = draw(seed, 0, ids, 0, RNG_INIT_POS)
    x = ((2 * u01_f32(r[0]).astype(np.float64) - 1) * half).astype(np.float32)
    y = ((2 * u01_f32(r[1]).astype(np.float64) - 1) * half).astype(np.float32)
    t = draw(seed, 0, ids, 0, RNG_INIT_ANGLE)
    th = ((2 * u01_f32(t[0]).astype(np.float64) - 1) * math.pi).astype(np.float32)
    return x, y, th


def star_trap_walls(n_hands=2, half_delta=0.3, r_big=15.0, r_small=6.0):
    """Segments of a star-shaped trap (Star_Trap_Initialization,
    shared/set-up.h:259-290): 3 n_hands end points (the tip at r_big, two
    inner points at r_small, rotated by 2 pi / n_hands per hand), each hand
    contributing two walls.  n_hands = 2 gives the 4 segments a closed box
    takes besides its own walls."""
    pts = [(r_big, 0.0)]
    a, b = (0.5 * 2 * math.pi / n_hands) - half_delta, (0.5 * 2 * math.pi / n_hands) + half_delta
    pts += [(r_small * math.cos(a), r_small * math.sin(a)), (r_small * math.cos(b), r_small * math.sin(b))]
    for i in range(3, 3 * n_hands):
        x, y = pts[i - 3]
        c, s = math.cos(2 * math.pi / n_hands), math.sin(2 * math.pi / n_hands)
        pts.append((c * x - s * y, s * x + c * y))
    walls = []
    for i in range(0, 3 * (n_hands - 1) + 1, 3):
        walls.append((*pts[i], *pts[i + 1]))
        walls.append((*pts[i + 2], *pts[(i + 3) % (3 * n_hands)]))
    return walls


def circle_config(n=4096, L=40.0, model=abi.MODEL_ABP, integrator=abi.INT_RK2, seed=6):
    """A circular box of radius L (the reference built with CIRCULAR_BOX and
    without PERIODIC_BOUNDARY_CONDITION, parallel/box.h:285-294): particles
    beyond r = L - 1 turn away from the circle.  ABP: the reference's R12 pair
    law and alignment; continuous: g = 1, alpha = 0."""
    p = reference_defaults(model)
    p.n, p.L, p.seed, p.integrator = n, L, seed, integrator
    p.boundary = abi.BOUNDARY_CIRCLE
    p.Dr, p.dt, p.skin = 0.1, 0.005, 0.3
    if model == abi.MODEL_CONTINUOUS:
        p.g, p.alpha, p.v0, p.dt = 1.0, 0.0, 0.5, 0.01
    return p


def circle_state(p, seed=None):
    """Particles on a square lattice of spacing 1.05 inside radius L - 1.2;
    random headings."""
    seed = p.seed if seed is None else seed
    g = np.arange(-p.L + 2.0, p.L - 2.0, 1.05)
    X, Y = np.meshgrid(g, g)
    x, y = X.ravel(), Y.ravel()
    keep = np.hypot(x, y) < p.L - 1.2
    x, y = x[keep][:p.n], y[keep][:p.n]
    if x.size < p.n:
        raise ValueError("circle too small for n particles")
    ids = np.arange(p.n, dtype=np.uint32)
    r = draw(seed, 0, ids, 0, RNG_INIT_ANGLE)
    th = ((2 * u01_f32(r[0]).astype(np.float64) - 1) * math.pi).astype(np.float32)
    return x.astype(np.float32), y.astype(np.float32), th


def walls_state(p, seed=None):
    """Particles on a square lattice of spacing 1.05 inside the box, at
    least 2 from the box walls and 1.6 from the extra segments; random
    headings."""
    seed = p.seed if seed is None else seed
    g = np.arange(-p.L + 2.0, p.L - 2.0, 1.05)
    X, Y = np.meshgrid(g, g)
    x, y = X.ravel(), Y.ravel()
    keep = np.ones(x.size, bool)
    for w in range(p.n_walls):
        x1, y1, x2, y2 = list(p.walls[w])
        ex, ey = x2 - x1, y2 - y1
        t = np.clip(((x - x1) * ex + (y - y1) * ey) / (ex * ex + ey * ey), 0.0, 1.0)
        keep &= np.hypot(x - (x1 + t * ex), y - (y1 + t * ey)) > 1.6
    x, y = x[keep][:p.n], y[keep][:p.n]
    if x.size < p.n:
        raise ValueError("box too small for n particles")
    ids = np.arange(p.n, dtype=np.uint32)
    r = draw(seed, 0, ids, 0, RNG_INIT_ANGLE)
    th = ((2 * u01_f32(r[0]).astype(np.float64) - 1) * math.pi).astype(np.float32)
    return x.astype(np.float32), y.astype(np.float32), th


def lyapunov_config(n=16384, rho=1.0, seed=3, integrator=abi.INT_RK4) -> abi.SppParams:
    """Continuous-time Vicsek for the Lyapunov spectrum: N = 16,384 at
    rho = 1 (L = 64), v0 = 0.5, g = 1, alpha = 0, D_r = 0, r = 1, RK4 with
    dt = 0.01 (ContinuousParticle, shared/particle.h:254-378, with RK4 in
    place of its Euler move)."""
    p = reference_defaults(abi.MODEL_CONTINUOUS)
    p.n, p.seed, p.integrator = n, seed, integrator
    p.L = 0.5 * math.sqrt(n / rho)
    p.v0, p.g, p.alpha, p.Dr, p.r_align, p.dt = 0.5, 1.0, 0.0, 0.0, 1.0, 0.01
    p.force_law = abi.FORCE_NONE
    p.skin = 0.3
    return p


def sweep_points(n_points=512, n_min=1024, n_max=65536, eta=(0.05, 0.6), rho=(0.25, 2.0),
                 v0=0.5, seed=4):
    """Parameter points of the batched Vicsek sweep: N log-uniform in
    [n_min, n_max], eta and rho uniform, L = sqrt(N) / (2 sqrt(rho)), v0 = 0.5,
    dt = 1; drawn from the Philox sweep stream (SPP_RNG_SWEEP = 7).  Returns
    one SppParams per point, system_id = index."""
    ids = np.arange(n_points, dtype=np.uint32)
    a = draw(seed, 0, ids, 0, 7)
    u = [u01_f32(w).astype(np.float64) for w in a]
    logn = np.log(n_min) + u[0] * (np.log(n_max) - np.log(n_min))
    N = np.floor(np.exp(logn)).astype(np.int64)
    etas = eta[0] + u[1] * (eta[1] - eta[0])
    rhos = rho[0] + u[2] * (rho[1] - rho[0])
    out = []
    for s in range(n_points):
        p = vicsek_config(n=int(N[s]), L=float(0.5 * math.sqrt(N[s] / rhos[s])), eta=float(etas[s]),
                          seed=seed)
        p.v0 = v0
        p.system_id = s
        out.append(p)
    return out


def sweep_state(points, seed=4):
    """Uniform positions / headings of every point, concatenated."""
    xs, ys, ts = [], [], []
    for p in points:
        x, y, th = random_state(p.n, p.L, seed=seed, system=p.system_id)
        xs.append(x)
        ys.append(y)
        ts.append(th)
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(ts)
