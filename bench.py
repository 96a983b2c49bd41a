"""Throughput of the per-step particle update on GB300.

Workload (one GPU): repulsive active Brownian / Vicsek particles, N =
1,048,576 disks of radius 0.5 in a periodic 1024 x 1024 box, harmonic
repulsion k(1 - r/2a) with k = 10, alignment torque (g/n_i) sum sin(theta_j -
theta_i) within r = 1, D_r = 0.1, v0 = 1, RK2 with dt = 0.005, Verlet skin
0.3, seeded uniform positions and headings.  One bench step = 200 simulation
steps (one replay of the captured step graphs); the default 50 timed bench
steps are the workload's 10,000 simulation steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  value = particle-steps/s over all ranks (each rank runs
an independent replica: the sweep-style "replicas only" multi-GPU mode).  At
one GPU the line also carries "sweep": sweep points/hour at |dP| <= 0.02
against full runs for the 512-point batched Vicsek sweep with the learned
surrogate, next to the same sweep without it and the plain GPU path run
point by point.
"""
import argparse
import ctypes as C
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s (N=1M Vicsek)"
UNIT = "particle-steps/s"
N_FULL = 1 << 20
L_FULL = 512.0
SIM_STEPS_PER_BENCH_STEP = 200
ALG_BYTES_PER_PARTICLE_STEP = 80  # RK2: stage 1 reads s0, writes s1/2; stage 2 reads s1/2, s0, writes s1


def workload_config(n):
    return {
        "workload": "repulsive ABP/Vicsek, N=1,048,576 disks a=0.5, periodic 1024x1024 box (L=512), "
                    "harmonic k=10, (g/n_i) sum sin alignment r=1, D_r=0.1, v0=1, RK2 dt=0.005, "
                    "Verlet skin 0.3, seed 1",
        "n": n,
        "sim_steps_per_bench_step": SIM_STEPS_PER_BENCH_STEP,
        "parallelism": "replicas (one independent system per GPU)",
        "l2": "flushed (256 MB write) between timed bench steps; within a bench step the "
              "~80 MB working set stays L2-resident, as in a production run",
    }


def dist_env():
    from spp_gb300.replicas import dist_env as env
    return env()


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 restatement (oracle/spp_oracle64.c) on host cores.
# ---------------------------------------------------------------------------
def _cpu_workload(workload, seed):
    """(params, FP64 state, advance(k, step)) of one full-size CPU replica."""
    import numpy as np
    from oracle import oracle as O
    from spp_gb300 import configs
    if workload == "abp":
        p = configs.abp_config(n=N_FULL, L=L_FULL, seed=seed)
        x, y, th = configs.random_state(p.n, p.L, seed=seed)
    elif workload == "vicsek":
        p = configs.vicsek_config(seed=seed)
        x, y, th = configs.random_state(p.n, p.L, seed=seed)
    elif workload == "vesicles":
        p = configs.vesicle_config(seed=seed)
        x, y, th = configs.vesicle_state(p)
    elif workload == "lyapunov":
        p = configs.lyapunov_config(seed=seed)
        x, y, th = configs.random_state(p.n, p.L, seed=seed)
    else:
        raise ValueError(workload)
    s = O.State64(x, y, th)
    if workload == "lyapunov":
        # the Benettin clone method of the reference (parallel/lyapunovbox.h:
        # 128-194): the base system and k = 8 perturbed clones, renormalised
        # every 10 steps
        V = np.random.default_rng(seed).standard_normal(3 * p.n * 8)

        def advance(k, step):
            O.lyap_clone64(p, s, V, max(1, k // 10), 10)
    else:
        def advance(k, step):
            O.run64(p, s, k, step0=step)
    return p, advance


def _cpu_worker(conn, workload, seed):
    sys.path.insert(0, str(ROOT))
    _, advance = _cpu_workload(workload, seed)
    step = 0
    conn.send("ready")
    while True:
        msg = conn.recv()
        if msg is None:
            break
        k = int(msg)
        t0 = time.perf_counter()
        advance(k, step)
        step += k
        conn.send(time.perf_counter() - t0)


class CpuPool:
    """One process per host core, each holding a full-size replica."""

    def __init__(self, cores, workload="abp"):
        ctx = mp.get_context("spawn")
        self.procs, self.conns = [], []
        for r in range(cores):
            a, b = ctx.Pipe()
            pr = ctx.Process(target=_cpu_worker, args=(b, workload, 1000 + r), daemon=True)
            pr.start()
            self.procs.append(pr)
            self.conns.append(a)
        for c in self.conns:
            assert c.recv() == "ready"

    def step(self, k):
        t0 = time.perf_counter()
        for c in self.conns:
            c.send(k)
        for c in self.conns:
            c.recv()
        return time.perf_counter() - t0

    def close(self):
        for c in self.conns:
            try:
                c.send(None)
            except Exception:
                pass
        for p in self.procs:
            p.join(timeout=10)


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_baseline(sim_steps=2, cores=None):
    cores = cores or cpu_cores()
    pool = CpuPool(cores)
    try:
        pool.step(1)  # warm-up: first-touch of the replicas
        wall = pool.step(sim_steps)
    finally:
        pool.close()
    value = cores * N_FULL * sim_steps / wall
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"FP64 restatement of the reference step (oracle/spp_oracle64.c), "
                      f"{cores} concurrent single-thread replicas x N=1,048,576 x {sim_steps} RK2 steps, "
                      f"{wall:.1f} s wall"}


# bounded CPU samples of the other configurations (steps per replica)
CPU_SAMPLE_STEPS = {"vicsek": 1000, "vesicles": 10, "lyapunov": 20}


def cpu_baseline_workload(workload, unit, cores=None):
    """The FP64 restatement of a configuration on every host core (one
    full-size replica per core), over CPU_SAMPLE_STEPS steps."""
    cores = cores or cpu_cores()
    k = CPU_SAMPLE_STEPS[workload]
    p, _ = _cpu_workload(workload, 0)
    pool = CpuPool(cores, workload)
    try:
        pool.step(min(k, 10))  # warm-up
        wall = pool.step(k)
    finally:
        pool.close()
    what = {"vicsek": "plain Vicsek steps", "vesicles": "RK4 steps of the vesicle system",
            "lyapunov": "RK4 steps of the base system and 8 clones (Benettin clone method, "
                        "oracle/spp_oracle64.c orc64_lyap_clone) from the disordered initial state "
                        "(shorter neighbour lists than the GPU's flocked window)"}[workload]
    return {"value": cores * p.n * k / wall, "unit": unit, "cores": cores, "kind": "port",
            "sample": f"FP64 restatement (oracle/spp_oracle64.c), {cores} concurrent single-thread "
                      f"replicas x N={p.n:,} x {k} {what}, {wall:.1f} s wall"}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(gpu_index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def ncu_traffic_per_launch(n, summary="k_abp_stage_abp1M_rk2.md"):
    """DRAM bytes per k_abp_stage launch from a committed ncu summary
    (profiles/<summary>, the line 'dram bytes per launch: <bytes> at
    n=<n>'), scaled to n particles."""
    f = ROOT / "profiles" / summary
    if not f.exists():
        return None
    import re
    m = re.search(r"dram bytes per launch:\s*([0-9.eE+]+)\s*at n=([0-9]+)", f.read_text())
    if not m:
        return None
    return float(m.group(1)) * n / float(m.group(2))


# ---------------------------------------------------------------------------
# sweep leg: 512-point batched Vicsek sweep with the learned surrogate
# ---------------------------------------------------------------------------
SWEEP_TOL = 0.02


def point_alone(p, x, y, th, max_steps=20000):
    """One sweep point through the plain single-system path (System +
    spp_step: the one-cluster kernel for small systems, the multi-kernel
    step otherwise): max_steps steps, the stationary P = mean of P over the
    second half, sampled every step."""
    import numpy as np
    from spp_gb300 import System
    half = max_steps // 2
    with System(p) as s:
        s.upload(x, y, th)
        s.step(max_steps - half)
        series, _, _ = s.polarization_series(half, every=1)
    return float(np.mean(series))


def sweep_leg(sample_points=64, seed=4):
    """Sweep points/hour at |dP| <= 0.02 against full runs: the batched
    sweep steered by the surrogate, the batched sweep without it, and the
    plain GPU path run point by point (each point alone through System +
    spp_step, run to the end; a seeded random sample of points stratified by
    size, the mean time per point extrapolated to all of them).  Points/hour
    count only the points answered within the tolerance."""
    import numpy as np
    from spp_gb300 import configs, surrogate

    pts = configs.sweep_points(seed=seed)
    n = len(pts)
    plain = surrogate.run_sweep(pts, use_surrogate=False, seed=seed)
    res = surrogate.run_sweep(pts, tol=SWEEP_TOL, seed=seed)
    err = np.abs(res.p_answer - plain.p_full)
    ran = np.isfinite(res.p_full)
    within = err <= SWEEP_TOL
    # point by point: a sample stratified by size (sample_points // 4 from each quartile of N)
    sizes = np.array([p.n for p in pts])
    order = np.argsort(sizes, kind="stable")
    rng = np.random.default_rng(seed)
    sample = np.concatenate([rng.choice(q, size=min(len(q), sample_points // 4), replace=False)
                             for q in np.array_split(order, 4)])
    x0, y0, t0s = configs.sweep_state(pts, seed=seed)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    per_point = []
    for s_ in sample:
        sl = slice(offs[s_], offs[s_ + 1])
        t0 = time.perf_counter()
        p_one = point_alone(pts[s_], x0[sl], y0[sl], t0s[sl])
        per_point.append(time.perf_counter() - t0)
        assert abs(p_one - plain.p_full[s_]) <= 1e-9, "a point run alone must reproduce its batched run"
    # equal counts from equal-sized quartiles: the sample mean estimates the sweep's mean
    mean_pp = float(np.mean(per_point))
    ret = res.retired
    pph = lambda count, wall: count / wall * 3600.0
    return {
        "metric": f"sweep points/hour at |dP|<={SWEEP_TOL} vs full runs",
        "workload": (f"{n} Vicsek points, N log-uniform [1024, 65536] (total {sum(p.n for p in pts):,} "
                     f"particles), eta U[0.05,0.6], rho U[0.25,2], v0=0.5, dt=1, 20,000 steps, "
                     f"stationary P over the second half; surrogate 7->128->128->1 GELU, BF16 weights, "
                     f"ensemble 5, Adam lr 1e-3, window 500 steps, 10% held out, seed {seed}"),
        "batched_surrogate": {"points_per_hour": pph(int(within.sum()), res.wall_s), "wall_s": res.wall_s,
                              "answered_within_tol": int(within.sum()),
                              "particle_steps": res.particle_steps, "retired": int(ret.sum()),
                              "rounds": res.rounds, "runs_s": res.timings["runs_s"],
                              "train_s": res.timings["train_s"], "phases": res.timings["phases"]},
        "batched_plain": {"points_per_hour": pph(n, plain.wall_s), "wall_s": plain.wall_s,
                          "particle_steps": plain.particle_steps},
        "point_by_point": {"points_per_hour": 3600.0 / mean_pp, "mean_s_per_point": mean_pp,
                           "sampled_points": int(len(sample)),
                           "sample": "seeded random sample stratified by N (equal counts per size quartile), "
                                     "each point run alone to 20,000 steps through System + spp_step (the "
                                     "one-cluster kernel where the system fits, else the multi-kernel step), "
                                     "P every step over the second half; mean time per point x all points"},
        "speedup_vs_point_by_point": (int(within.sum()) / res.wall_s) / (1.0 / mean_pp),
        "speedup_vs_batched_plain": (int(within.sum()) / res.wall_s) / (n / plain.wall_s),
        "accuracy": {"retired_within_tol_frac": float(np.mean(err[ret] <= SWEEP_TOL)) if ret.any() else None,
                     "retired_err_median": float(np.median(err[ret])) if ret.any() else None,
                     "retired_err_max": float(np.max(err[ret])) if ret.any() else None,
                     "all_points_within_tol_frac": float(np.mean(within)),
                     "heldout_err_median": float(np.median(res.heldout_err)),
                     "heldout_within_tol_frac": float(np.mean(res.heldout_err <= SWEEP_TOL)),
                     "full_runs_bitexact": bool(np.array_equal(res.p_full[ran], plain.p_full[ran]))},
    }


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    ws, rank, local = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np
    import torch
    from spp_gb300 import System, configs

    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
    n = N_FULL
    p = configs.abp_config(n=n, L=L_FULL, seed=1 + rank)
    x, y, th = configs.random_state(n, L_FULL, seed=1 + rank)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    S = SIM_STEPS_PER_BENCH_STEP
    with System(p) as s:
        s.upload(x, y, th)
        for _ in range(args.warmup):
            s.step(S)
        s.sync()
        # the state entering the timed region: the end-to-end leg replays the
        # same trajectory through host buffers
        def pinned_state():
            return tuple(torch.empty(n, dtype=dt).pin_memory().numpy()
                         for dt in (torch.float32, torch.float32, torch.float32, torch.int32, torch.int32))
        buf_in, buf_out = pinned_state(), pinned_state()
        s.download(out=buf_in)
        step_at = s.step0 + int(s.observables().step)
        launches0 = s.kernel_launches()
        regrow0 = int(s.observables().list_regrowths)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local if ws > 1 else int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0))
        times = []
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            times.append(s.time_steps(S))
        wall = time.perf_counter() - wall0
        clocks = sampler.stop()
        torch.cuda.synchronize()
        launches = s.kernel_launches() - launches0
        # spp_time_steps times list-overflow recoveries too; count them
        overflows = int(s.observables().list_regrowths) - regrow0
        elapsed_ms = sum(times)
        if dist:
            from spp_gb300.replicas import max_over_ranks
            elapsed_ms = max_over_ranks(elapsed_ms, dist)   # the slowest rank sets the wall time
            dist.barrier()
        obs = s.observables()
        # kernel-level timing for the roofline: CUDA events around every stage kernel
        prof = s.profile(200)
        stage_avg_ms = prof.stage_ms / max(1, prof.stage_launches)
        rebuild_avg_ms = prof.rebuild_ms / max(1, prof.rebuilds)

        # end to end through the C ABI with host buffers (pinned), copies inside:
        # the host holds the trajectory between chunks of S steps and each
        # chunk uploads the state the previous one downloaded, starting from
        # the state that entered the timed region; the steps are bit-exact, so
        # this is the timed region's own trajectory, chunk for chunk
        e2e_times = []
        for k in range(0 if args.no_e2e else args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.upload(buf_in[0], buf_in[1], buf_in[2], step0=step_at, img_x=buf_in[3], img_y=buf_in[4])
            s.step(S)
            s.download(out=buf_out)
            e2e_times.append(time.perf_counter() - t0)
            buf_in, buf_out = buf_out, buf_in
            step_at += S
        e2e_value = n * S * len(e2e_times) / sum(e2e_times) if e2e_times else None
    value = ws * n * S * args.steps / (elapsed_ms / 1e3)
    peak, peak_kind = measured_hbm_peak()
    achieved = ALG_BYTES_PER_PARTICLE_STEP / 2 * n / (stage_avg_ms / 1e3) / 1e9
    traffic = ncu_traffic_per_launch(n)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: Philox-seeded uniform positions and headings (no dataset involved)",
        "config": workload_config(n),
        "ms_per_sim_step": elapsed_ms / args.steps / S,
        "gpu_launches": int(launches),
        "overflows_in_timed_region": overflows,
        "clocks": clocks,
        "wall_s_timed_region": wall,
        "roofline": {
            "bound": "hbm", "kernel": "k_abp_stage (force gather + RK2 stage)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "alg_bytes_per_launch": ALG_BYTES_PER_PARTICLE_STEP // 2 * n,
            "avg_launch_ms": stage_avg_ms,
            "traffic": traffic,
            "note": "state (~80 MB) is L2-resident between steps, so achieved is an effective "
                    "bandwidth over algorithmic bytes; traffic is DRAM bytes per launch from ncu",
        },
        "rebuild": {"avg_ms": rebuild_avg_ms, "per_200_steps": prof.rebuilds},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 20 * n,
                "d2h_bytes_per_step": 20 * n,
                "path": "spp_upload_state (pinned host: x, y, theta, image counters) + spp_step(200) + "
                        "spp_download_state (pinned host) per bench step, host wall clock; the timed "
                        "region's trajectory replayed chunk by chunk from its entry state"},
        "observables": {"polarization": obs.polarization, "rebuilds": obs.n_rebuilds,
                        "max_neighbors": obs.max_neighbors, "list_capacity": obs.list_capacity},
    }
    if rank == 0 and ws == 1 and not args.no_sweep:
        line["sweep"] = sweep_leg()
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sim_steps=2)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU path (its FP64 restatement) on host cores
# ---------------------------------------------------------------------------
def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    cores = cpu_cores()
    pool = CpuPool(cores)
    try:
        for _ in range(args.warmup):
            pool.step(1)
        walls = [pool.step(1) for _ in range(args.steps)]
    finally:
        pool.close()
    total = sum(walls)
    value = cores * N_FULL * args.steps / total
    sample = (f"each bench step: {cores} concurrent single-thread replicas (one per host core) x "
              f"N=1,048,576 x 1 RK2 step of the FP64 restatement (oracle/spp_oracle64.c); the "
              f"reference's own code cannot run here: it is header-only C++ that needs GSL and "
              f"MPI, and its source checkout, from which the harness is compiled, is not on "
              f"this machine")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: Philox-seeded uniform positions and headings",
        "config": workload_config(N_FULL),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# the other configurations (one JSON line each; not the headline)
# ---------------------------------------------------------------------------
def sweep_sharded(args):
    """The 512-point sweep with the surrogate over N GPUs (torchrun): points
    split by cost, each rank runs its shard, surrogate fits use every rank's
    completed points; points/hour over the slowest rank's wall time."""
    import numpy as np
    import torch.distributed as dist
    from spp_gb300 import configs, replicas
    ws, rank, local = dist_env()
    os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist.init_process_group("gloo")   # host-side exchange of small arrays
    pts = configs.sweep_points(n_points=512)
    dist.barrier()
    t0 = time.perf_counter()
    ans, full, ret, res = replicas.run_sweep_sharded(pts, rank, ws, replicas.Exchange(dist), max_steps=20000,
                                                     window=500, seed=4)
    wall = replicas.max_over_ranks(time.perf_counter() - t0, dist)
    if rank == 0:
        print(json.dumps({"metric": "sweep points/hour at |dP|<=0.02 vs full runs", "workload": "sweep",
                          "value": len(pts) / wall * 3600.0, "unit": "points/hour", "n_gpus": ws,
                          "higher_is_better": True, "scaling": "strong", "data": "synthetic",
                          "config": {"workload": "512 Vicsek points (N log-uniform [1024, 65536]), 20,000 steps, "
                                                 "surrogate sweep sharded by cost over the ranks"},
                          "wall_s": wall, "retired": int(ret.sum()),
                          "answered": int(np.isfinite(ans).sum())}), flush=True)
    dist.destroy_process_group()


def other_workload(args):
    """Throughput of configurations 1, 3, 4 and 5 on one GPU: plain Vicsek
    N=4096 (32 B/particle-step), vesicles with swimmers (163,840 bodies, RK4,
    ~260 B/body-step), the Lyapunov spectrum (N=16,384, k=8 tangent vectors,
    ~2,550 B/particle-step) and the 512-point sweep.  Effective bandwidth =
    algorithmic bytes x rate (the working sets are L2-resident)."""
    import numpy as np
    import torch
    from spp_gb300 import System, configs

    peak, peak_kind = measured_hbm_peak()
    w = args.workload
    if w == "batch64":
        # the small case the kernel captures use: 64 sweep points stepped 40
        # times, then 60 surrogate training iterations on 300 samples
        from spp_gb300 import Batch, surrogate
        pts = configs.sweep_points(n_points=64)
        x, y, th = configs.sweep_state(pts, seed=4)
        with Batch(pts) as b:
            b.set_windows(500, 10000, 20000)
            b.upload(x, y, th)
            ms = b.time_steps(40)
        rng = np.random.default_rng(0)
        f = rng.standard_normal((300, 7)).astype(np.float32)
        t = rng.uniform(0, 1, 300).astype(np.float32)
        mlp = surrogate.Mlp(5, 7, 4)
        t0 = time.perf_counter()
        mlp.train(f, t, iters=60, lr=1e-3)
        train_ms = (time.perf_counter() - t0) * 1e3
        mlp.close()
        n = sum(p.n for p in pts)
        print(json.dumps({"metric": "particle-steps/s", "workload": "batch64", "value": n * 40 / (ms / 1e3),
                          "unit": "particle-steps/s", "n_gpus": 1, "ms_per_step": ms / 40,
                          "config": {"workload": f"64 sweep points ({n:,} particles), 40 steps; "
                                                 "60 training iterations of the 5-member surrogate on 300 samples"},
                          "train_ms_per_iteration": train_ms / 60}), flush=True)
        return
    if w == "stage262k":
        # the small case of the headline model for full kernel captures: the
        # same density at a quarter of the particles, 100 steps from the
        # random start, 200 steps of direct launches timed kernel by kernel
        # (spp_profile, which a profiler sees), then --steps x 200 graph steps
        n, L = 262144, 256.0
        p = configs.abp_config(n=n, L=L, seed=1)
        x, y, th = configs.random_state(n, L, seed=1)
        with System(p) as s:
            s.upload(x, y, th)
            s.step(100)
            s.sync()
            pr = s.profile(200)
            ms = [s.time_steps(200) for _ in range(max(1, args.steps))]
            o = s.observables()
        stage_us = pr.stage_ms / max(1, pr.stage_launches) * 1e3
        achieved = 40.0 * n / (stage_us * 1e-6) / 1e9
        print(json.dumps({"metric": "particle-steps/s", "workload": "stage262k",
                          "value": n * 200 / (min(ms) / 1e3), "unit": "particle-steps/s", "n_gpus": 1,
                          "ms_per_sim_step": min(ms) / 200, "stage_us": stage_us,
                          "rebuild_us": pr.rebuild_ms / max(1, pr.rebuilds) * 1e3, "rebuilds_per_200": pr.rebuilds,
                          "max_neighbors": o.max_neighbors, "list_capacity": o.list_capacity,
                          "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                       "frac": achieved / peak, "alg_bytes_per_unit": 40},
                          "config": {"workload": "repulsive ABP with the headline parameters at N=262,144, L=256 "
                                                 "(the same density), 100 steps in"}}), flush=True)
        return
    if w == "mlp":
        # the surrogate's training iteration (5 members, 7 -> 128 -> 128 -> 1,
        # 300 samples) with the tensor-core kernels and with the scalar ones
        from spp_gb300 import surrogate
        rng = np.random.default_rng(1)
        f = rng.standard_normal((300, 7)).astype(np.float32)
        t = (0.5 + 0.3 * np.tanh(f[:, 0])).astype(np.float32)
        iters = 50 * max(1, args.steps)
        out = {}
        for scalar in ("0", "1"):
            os.environ["SPP_MLP_SCALAR"] = scalar
            mlp = surrogate.Mlp(ensemble=5, seed=4)
            mlp.train(f, t, iters=100)
            t0 = time.perf_counter()
            loss = mlp.train(f, t, iters=iters)
            out["scalar" if scalar == "1" else "tensor_cores"] = {
                "us_per_iteration": (time.perf_counter() - t0) / iters * 1e6,
                "final_loss": [float(v) for v in loss]}
            mlp.close()
        os.environ.pop("SPP_MLP_SCALAR", None)
        print(json.dumps({"metric": "us per training iteration", "workload": "mlp",
                          "value": out["tensor_cores"]["us_per_iteration"], "unit": "us",
                          "higher_is_better": False, "iterations": iters, **out,
                          "config": {"workload": "5-member ensemble, 7 -> 128 -> 128 -> 1, 300 samples, Adam; "
                                                 "host wall clock around Mlp.train after 100 warm iterations"}}),
              flush=True)
        return
    if w == "sweep" and dist_env()[0] > 1:
        sweep_sharded(args)
        return
    if w == "sweep":
        line = {"metric": "sweep points/hour at |dP|<=0.02 vs full runs", "n_gpus": 1, "data": "synthetic"}
        line.update(sweep_leg())
        line["value"] = line["batched_surrogate"]["points_per_hour"]
        line["unit"] = "points/hour"
        line["higher_is_better"] = True
        print(json.dumps(line), flush=True)
        return
    if w == "vicsek":
        p = configs.vicsek_config()
        x, y, th = configs.random_state(p.n, p.L, seed=0)
        chunk, alg, unit = 2000, 32, "particle-steps/s"
        desc = "plain Vicsek (arg-sum rule), N=4096, L=32, v0=0.5, r=1, eta=0.3, dt=1, 2000 steps per bench step"
    elif w == "vesicles":
        p = configs.vesicle_config()
        x, y, th = configs.vesicle_state(p)
        chunk, alg, unit = 200, 260, "body-steps/s"
        desc = ("1024 ring vesicles x 128 beads + 32 swimmers each (163,840 bodies), bonds k=100, bending "
                "kappa=10, WCA-like R12, RK4 dt=0.002, L=1081 (30% area fraction by enclosed area); 200 "
                "steps per bench step")
    elif w == "lyapunov":
        p = configs.lyapunov_config()
        x, y, th = configs.random_state(p.n, p.L, seed=3)
        chunk, alg, unit = 100, 2550, "particle-steps/s"
        desc = ("continuous Vicsek N=16,384, L=64, RK4 dt=0.01, k=8 tangent vectors, linearised RK4, "
                "FP64 Gram-Schmidt every 10 steps; 100 steps per bench step, timed after a 2000-step pre-run")
    else:
        raise SystemExit(f"unknown workload {w}")
    with System(p) as s:
        s.upload(x, y, th)
        times = []
        if w == "lyapunov":
            s.lyap_init(8, seed=3)
            # the noise-free model flocks and its neighbour lists grow over the
            # first ~2000 steps; the timed window is the steady part of a long run
            s.lyap_step(2000, renorm_every=10)
            for _ in range(args.warmup):
                s.lyap_step(chunk, renorm_every=10)
            s.sync()
            for _ in range(args.steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s.lyap_step(chunk, renorm_every=10)
                s.sync()
                times.append((time.perf_counter() - t0) * 1e3)
            lam, T = s.lyap_exponents()
            extra = {"lyapunov_exponents": [float(v) for v in lam], "time_span": T,
                     "timing": "host wall clock around spp_lyap_step + spp_sync"}
        else:
            for _ in range(args.warmup):
                s.step(chunk)
            s.sync()
            for _ in range(args.steps):
                times.append(s.time_steps(chunk))
            extra = {"timing": "CUDA events on the system's stream (spp_time_steps)",
                     "polarization": s.observables().polarization}
    ms = float(np.sum(times))
    value = p.n * chunk * args.steps / (ms / 1e3)
    achieved = alg * value / 1e9
    line = {"metric": unit, "workload": w, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "ms_per_sim_step": ms / args.steps / chunk,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (Philox-seeded)",
            "config": {"workload": desc, "n": int(p.n)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "alg_bytes_per_unit": alg,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "note": "effective bandwidth of the whole step; working set L2-resident"}}
    if w == "vesicles":
        line["roofline"]["traffic"] = ncu_traffic_per_launch(p.n, "k_abp_stage_vesicles163k_rk4.md")
        line["roofline"]["traffic_note"] = "cold-cache DRAM bytes per k_abp_stage launch (ncu, 4 stages per step)"
    line.update(extra)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_workload(w, unit)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-sweep", action="store_true", help="skip the 512-point sweep leg")
    ap.add_argument("--workload", default="abp",
                    choices=["abp", "vicsek", "vesicles", "lyapunov", "sweep", "batch64", "stage262k", "mlp"],
                    help="abp: the headline line (default); the others print their own line")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "abp":
        other_workload(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
