"""Long-run statistical parity (config-1 Vicsek, N = 4096, eta = 0.3,
dt = 1): discrete Vicsek is chaotic, so the FP32 device run and the FP64
restatement decorrelate within tens of steps; they must sample the same
stationary state.  Compared after a 500-step transient over 1500 steps:
<P> within the autocorrelation-corrected error bars of both series
(analyze/statistics.h:68-82), both Binder forms within block-scatter error
bars, and g(r) within the frame-to-frame scatter."""
import numpy as np
import pytest

from oracle import analysis_oracle as A
from oracle import oracle as O
from spp_gb300 import System, configs, observables

pytestmark = pytest.mark.gpu

T0, T = 500, 2000
FRAMES = range(T0 + 100, T + 1, 100)


def block_binder(p, blocks=5):
    vals = []
    for b in np.array_split(np.asarray(p), blocks):
        st = observables.order_parameters(b, 1.0)
        vals.append((st["binder"], st["binder_reference"]))
    vals = np.array(vals)
    return vals.mean(0), vals.std(0, ddof=1) / np.sqrt(blocks)


def test_vicsek_long_run_statistics_match_fp64(gpu_lib):
    p = configs.vicsek_config()
    x, y, th = configs.random_state(p.n, p.L, seed=0)
    # device: P every step, g(r) every 100 steps
    gpu_p, gpu_g = [], []
    with System(p) as s:
        s.upload(x, y, th)
        for t0 in range(0, T, 100):
            pp, _, _ = s.polarization_series(100, every=1)
            gpu_p.extend(pp)
            if t0 + 100 in FRAMES:
                gpu_g.append(s.radial_distribution(4.0, 20).astype(np.float64))
    # FP64 restatement: P every step, g(r) on the same frames
    st = O.State64(x, y, th)
    cpu_p, cpu_g = [], []
    for t in range(T):
        O.run64(p, st, 1, step0=t)
        cpu_p.append(A.frame_polarization(st.th))
        if t + 1 in FRAMES:
            cpu_g.append(A.radial_counts(st.x, st.y, p.L, 4.0, 20).astype(np.float64))
    a = observables.order_parameters(np.array(gpu_p[T0:]), 4 * p.L * p.L)
    b = observables.order_parameters(np.array(cpu_p[T0:]), 4 * p.L * p.L)
    # the trajectories did decorrelate (the comparison is statistical)
    assert np.max(np.abs(np.array(gpu_p[T0:]) - np.array(cpu_p[T0:]))) > 1e-3
    tol = 4.0 * np.hypot(a["error"], b["error"]) + 1e-3
    assert abs(a["mean"] - b["mean"]) < tol, (a["mean"], b["mean"], tol)
    (ga, gra), (ea, era) = block_binder(gpu_p[T0:])
    (gb, grb), (eb, erb) = block_binder(cpu_p[T0:])
    assert abs(ga - gb) < 4.0 * np.hypot(ea, eb) + 1e-3
    assert abs(gra - grb) < 4.0 * np.hypot(era, erb) + 1e-3
    # g(r): mean over frames, error from the frame-to-frame scatter
    G1, G2 = np.array(gpu_g), np.array(cpu_g)
    diff = G1.mean(0) - G2.mean(0)
    err = np.sqrt(G1.var(0, ddof=1) / len(G1) + G2.var(0, ddof=1) / len(G2))
    print("g(r) |diff| / err per bin:", np.round(np.abs(diff) / np.maximum(err, 1e-300), 2))
    assert np.all(np.abs(diff) <= 5.0 * err), np.abs(diff) / err
