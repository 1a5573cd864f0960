#!/usr/bin/env python
"""Benchmark of the GB300 2-opt engine on the single large instance.

Workload (one "step" = one best-improvement 2-opt move of a descent: the full
sweep over (n-2)(n-3)/2 pairs, the device argmin and the device reversal):
n = 100,000 cities from a seeded Gaussian mixture (200 clusters, sigma = 1% of
the [0,1e6)^2 box, float32), nearest-neighbour start tour, descent moves on
the device-resident tour.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is pair-evaluations per second over the K timed
steps (device time from CUDA events on the library's stream, L2 flushed
between steps); `e2e` is the same metric through the C-ABI call with host
buffers (logo_descend, one move per call: route H2D, move, route D2H).
Under torchrun every rank runs an independent replica (the path has no
cross-GPU exchange), and rank 0 prints the aggregate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "logo-tsp-solver_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

import instances  # noqa: E402
import logo_gpu as lg  # noqa: E402

SMS = 152           # GB300 streaming multiprocessors
LANES = 128         # FP32/INT32 lanes per SM per clock
OPS_PER_PAIR = 10   # algorithmic FP32 (6) + INT (4) ops per pair evaluation
METRIC = "2-opt pair-evals/s"
UNIT = "pair-evals/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=100000)
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--e2e-steps", type=int, default=40)
    p.add_argument("--cpu-sweeps", type=int, default=2)
    p.add_argument("--batched", type=int, default=1, help="include the batched comparison")
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--batch-kicks", type=int, default=200)
    p.add_argument("--batch-seed", type=int, default=3)
    p.add_argument("--plain-sample", type=int, default=32)
    return p.parse_args()


def workload(n, seed):
    xy = instances.clustered(n, seed, side=1.0e6, clusters=200, sigma_frac=0.01)
    route = lg.nn_tour(xy, 0)
    return xy, route


def pairs_per_sweep(n):
    return (n - 2) * (n - 3) // 2


def config(n, world, host=False):
    c = {
        "workload": f"single large instance: n={n} Gaussian mixture (200 clusters, "
                    "sigma=1% of [0,1e6)^2, fp32), nearest-neighbour start tour, "
                    "best-improvement 2-opt descent moves",
        "n": n,
        "step": "one full sweep + argmin + reversal" + (" on the host" if host else
                                                         " on the device"),
        "parallelism": "host threads" if host else (f"replicas x{world}" if world > 1
                                                     else "single GPU"),
    }
    if not host:
        c["l2"] = "flushed between timed steps (256 MiB write); inputs 1.6 MB"
    return c


# ----------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons (200 ms)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.idx)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "samples": len(sm), "power_w_max": max(power), "reasons": sorted(reasons)}


def gpu_index(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        parts = [p for p in vis.split(",") if p.strip()]
        if local_rank < len(parts):
            return parts[local_rank].strip()
    return str(local_rank)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# sweep kernel per LOGO_SWEEP_* variant: (kernel, screen)
SWEEP_KERNELS = {0: ("sweep_kernel", "MUFU screen"),
                 4: ("sweep_kernel5", "fused two-stage square-root-free screen"),
                 5: ("sweep_kernel6", "local-coordinate expanded screen"),
                 6: ("sweep_boxed_kernel", "boxed screen: row-block and window bounding "
                                           "boxes, then the local-coordinate screen")}
# kernels per sweep launch: the boxed variant runs window_stats_kernel and tile_filter_kernel first
SWEEP_LAUNCHES = {6: 3}


def profile_traffic(kernel):
    """DRAM bytes per sweep launch at n=100k from the committed ncu summary
    of that kernel (None if there is none)."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_n100k.md")
    try:
        with open(p) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_launch:"):
                    return float(ln.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


# ----------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(a, world, rank, local, dist):
    import torch
    lg.load()
    n = a.n
    xy, route = workload(n, a.seed + rank)
    pairs = pairs_per_sweep(n)
    s = lg.Solver(xy, device=local)
    s.set_route(route)
    s.begin_descent(0)
    ext = torch.cuda.ExternalStream(s.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    for _ in range(a.warmup):
        s.enqueue_sweep()
        s.enqueue_apply()
    s.sync()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(a.steps)]
    barrier(dist)
    torch.cuda.synchronize()
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    time.sleep(0.4)
    t_wall = time.perf_counter()
    for k in range(a.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        ev[k][0].record(ext)
        s.enqueue_sweep()
        ev[k][1].record(ext)
        s.enqueue_apply()
        ev[k][2].record(ext)
    s.sync()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    barrier(dist)
    sweep_ms = [e[0].elapsed_time(e[1]) for e in ev]
    step_ms = [e[0].elapsed_time(e[2]) for e in ev]
    moves, converged = s.progress()
    if converged or moves != a.warmup + a.steps:
        raise RuntimeError(f"descent ended early ({moves} moves); pick fewer steps")
    total_s = reduce_max(dist, sum(step_ms) / 1e3)
    value = world * pairs * a.steps / total_s
    ms_per_step = total_s * 1e3 / a.steps

    # e2e: the C-ABI call with host buffers, one move per call
    cur = s.get_route()
    buf = np.empty(n, dtype=np.uint32)
    for _ in range(3):
        cur, _ = s.optimize(cur, max_moves=1, stats=False, out=buf)
        cur = cur.copy()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        s.optimize(cur, max_moves=1, stats=False, out=buf)
        cur, buf = buf, cur
    e2e_s = reduce_max(dist, time.perf_counter() - t0)
    e2e = {"value": world * pairs * a.e2e_steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n + 2 * 128,
           "call": "logo_descend(max_moves=1) per step: route H2D, sweep, argmin, "
                   "reversal, route D2H"}

    # roofline of the sweep kernel (the dominant kernel)
    info = s.info()
    kname, screen = SWEEP_KERNELS[info["variant"]]
    peaks = measured_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    mean_sweep_s = statistics.mean(sweep_ms) / 1e3
    achieved_pairs = pairs / mean_sweep_s
    peak_ops = SMS * LANES * sm_max * 1e6
    roof = {
        "bound": "alu",
        "achieved": round(achieved_pairs * OPS_PER_PAIR / 1e12, 3),
        "peak": round(peak_ops / 1e12, 3),
        "unit": "TFLOP/s",
        "frac": round(achieved_pairs * OPS_PER_PAIR / peak_ops, 4),
        "traffic": profile_traffic(kname),
        "kernel": ("logo::window_stats_kernel + logo::tile_filter_kernel + "
                   if SWEEP_LAUNCHES.get(info["variant"]) else "")
                  + f"logo::{kname}<{info['rows_per_thread']},{info['warps_per_cta']}> "
                  f"({screen}, {info['tile_cols']}-column tiles; timed together)",
        "ops_per_pair": "6 FP32 + 4 INT (algorithmic convention, 1 distance/pair)",
        "peak_source": f"152 SMs x 128 FP32/INT32 lanes x sm_max_mhz={sm_max:g} "
                       "(MEASURED_PEAKS.json)",
        "achieved_pairs_per_s": achieved_pairs,
        "sweep_ms_mean": round(statistics.mean(sweep_ms), 4),
        "note": "achieved counts every pair of the sweep as decided; the screens decide "
                "most pairs without per-pair arithmetic (the boxed screen closes whole "
                "rows x 32-column blocks by a bounding-box test), always returning the "
                "reference's move, so frac above 1 measures pruning, not lane throughput; "
                "thread instructions per pair and issue-slot use are in profiles/",
    }
    if clocks.get("sm_mhz"):
        roof["frac_at_sampled_clock"] = round(
            achieved_pairs * OPS_PER_PAIR / (SMS * LANES * clocks["sm_mhz"] * 1e6), 4)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded Gaussian mixture, no dataset)",
        "config": config(n, world), "roofline": roof, "e2e": e2e, "clocks": clocks,
        "gpu_launches": (SWEEP_LAUNCHES.get(info["variant"], 1) + 1) * a.steps,
        "wall_s_timed_region": round(t_wall, 3),
    }

    if a.batched and rank == 0:
        out["batched"] = run_batched(a, local)

    # CPU baseline: the oracle's multi-threaded sweep on this host (rank 0)
    if rank == 0 and a.cpu_sweeps > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        threads = os.cpu_count() or 1
        cur = s.get_route()
        gpu_move = s.sweep_resident()
        t0 = time.perf_counter()
        key = None
        for _ in range(a.cpu_sweeps):
            key = oracle.best_move_key(xy, cur, threads=threads)
        cpu_s = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": pairs * a.cpu_sweeps / cpu_s, "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{a.cpu_sweeps} full sweeps of the same n={n} tour, oracle "
                      f"(per-edge nint, reference loop order) on {threads} threads",
            "same_move_as_gpu": oracle.unpack_key(key) == gpu_move,
        }
    s.close()
    return out


def run_batched(a, device):
    """Batched workload: 4096 instances, n log-uniform in [50, 2000], uniform
    float32 coordinates in [0,1e4)^2, random start tours, descent + 200
    segment kicks each, solved in one persistent launch per tile shape (one
    CUDA graph); against looping the plain single-instance path (logo_ils)
    over a stratified sample of the same instances, with identical final
    lengths required on that sample."""
    count, kicks = a.batch_count, a.batch_kicks
    coords, routes, seeds = instances.batched_workload(count, a.batch_seed)
    ns = np.array([len(r) for r in routes], dtype=np.int64)
    pairs = (ns - 2) * (ns - 3) // 2
    cache = os.path.join(PKG, "autotune_cache.json")
    with lg.Batch(count, int(ns.sum()), device=device) as b:
        # autotune on a stratified sample (reuses a cached table for this GPU)
        order = np.argsort(ns)
        tsample = order[np.linspace(0, count - 1, min(count, 256)).astype(int)]
        t0 = time.perf_counter()
        b.autotune([coords[k] for k in tsample], [routes[k] for k in tsample],
                   [seeds[k] for k in tsample], kicks=10, cache_path=cache, reuse=True)
        tune_s = time.perf_counter() - t0
        shapes = {str(n): b.shape_for(n) for n in (100, 300, 800, 1500)}
        b.solve(coords[:64], routes[:64], seeds[:64], kicks=2)  # warm-up
        got, res, ms = b.solve(coords, routes, seeds, kicks=kicks)
    sweeps = np.array([r["sweeps"] for r in res], dtype=np.int64)
    batched = count * (kicks + 1) / (ms / 1e3)
    # plain: the single-instance path, one instance at a time
    psample = order[np.linspace(0, count - 1, a.plain_sample).astype(int)]
    identical = True
    t0 = time.perf_counter()
    for k in psample:
        with lg.Solver(coords[k], device=device) as s:
            r, st = s.ils(routes[k], kicks, seeds[k], lg.KICK_SEGMENT)
        identical &= (st["final_length"] == res[k]["best_length"]) and bool(
            np.array_equal(r, got[k]))
    plain_s = time.perf_counter() - t0
    plain = len(psample) * (kicks + 1) / plain_s
    return {
        "workload": f"{count} instances, n log-uniform in [50,2000], uniform fp32 in "
                    f"[0,1e4)^2, random start, descent + {kicks} segment kicks each",
        "metric": "local-opts/s", "value": batched, "device_s": ms / 1e3,
        "pair_evals_per_s": float((sweeps * pairs).sum() / (ms / 1e3)),
        "moves": int(sum(r["moves"] for r in res)),
        "plain": {"value": plain, "unit": "local-opts/s", "sample": int(len(psample)),
                  "wall_s": plain_s,
                  "how": "logo_ils per instance (context create + ILS), stratified by n"},
        "speedup_vs_plain": batched / plain,
        "identical_lengths_and_tours_on_sample": bool(identical),
        "autotuned_shapes": shapes, "autotune_s": tune_s,
    }


def run_reference(a, rank):
    """The reference CPU path on the host cores: the oracle port of
    CPUMTSolver::optimizeStep + the move application, all threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    n = a.n
    xy = instances.clustered(n, a.seed, side=1.0e6, clusters=200, sigma_frac=0.01)
    route, _ = oracle.nn_tour(xy)
    threads = os.cpu_count() or 1
    pairs = pairs_per_sweep(n)

    def step(r):
        key = oracle.best_move_key(xy, r, threads=threads)
        d, i, j = oracle.unpack_key(key)
        return oracle.apply_move(r, i, j) if d < 0 else r

    r = route
    t0 = time.perf_counter()
    r = step(r)
    per = time.perf_counter() - t0
    # each timed step is a full sweep; bound the run to ~2 minutes
    budget = 120.0
    steps = max(1, min(a.steps, int(budget / max(per, 1e-3))))
    warm = min(a.warmup, 2)
    for _ in range(warm):
        r = step(r)
    t0 = time.perf_counter()
    for _ in range(steps):
        r = step(r)
    el = time.perf_counter() - t0
    value = pairs * steps / el
    sample = (f"{steps} descent steps (full {n}-city sweep + move) of the benchmark "
              f"workload on {threads} threads")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": steps, "warmup": warm, "ms_per_step": el * 1e3 / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Gaussian mixture, no dataset)",
        "config": config(n, 1, host=True),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    a = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if a.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(a, rank)), flush=True)
        return
    world, rank, local, dist = dist_setup()
    out = run_ours(a, world, rank, local, dist)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
