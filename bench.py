#!/usr/bin/env python
"""Benchmark of the GB300 2-opt engine.

Headline workload (one "step" = one best-improvement 2-opt move of a descent:
the full sweep over (n-2)(n-3)/2 pairs, the device argmin and the device
reversal): n = 100,000 cities from a seeded Gaussian mixture (200 clusters,
sigma = 1% of the [0,1e6)^2 box, float32), nearest-neighbour start tour,
descent moves on the device-resident tour.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is pairs decided per second over the K timed
steps (device time from CUDA events on the library's stream, L2 flushed
between steps): every pair of a sweep counts, whether the screen evaluated it
on its own or ruled it out with its block; the chosen move is the
reference's either way.  `e2e` is the same metric through the C-ABI call with
host buffers (logo_descend, one move per call: route H2D, move, route D2H).
`roofline` puts the sweep's executed lane operations (thread instructions
per sweep from the ncu capture of this command, in profiles/) over its live
duration against the lanes' peak; the pruning-inclusive figure is reported
beside it under its own name.  Further blocks: `dense` (the local-coordinate
screen, every pair screened on its own), `sweep_per_n` (one sweep of uniform
points on random tours at n = 10k, 100k, 1M), `large` (the n = 100k instance:
descent + 1000 double-bridge kicks), `batched` (4096 instances in one
persistent launch vs the single-instance path) and `serving` (Poisson request
stream, continuous batching vs one request at a time).
Under torchrun every rank runs an independent replica (the path has no
cross-GPU exchange), and rank 0 prints the aggregate.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "logo-tsp-solver_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import instances  # noqa: E402
import logo_gpu as lg  # noqa: E402

SMS = 152           # GB300 streaming multiprocessors
LANES = 128         # FP32/INT32 lanes per SM per clock
OPS_PER_PAIR = 10   # convention: FP32 (6) + INT (4) ops per pair evaluation
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
    p.add_argument("--dense", type=int, default=1, help="time the every-pair local screen")
    p.add_argument("--sweep-sizes", default="10000,100000,1000000",
                   help="sweep_per_n block sizes ('' to skip)")
    p.add_argument("--large-kicks", type=int, default=1000,
                   help="large block: double-bridge kicks after the descent (0 to skip)")
    p.add_argument("--batched", type=int, default=1, help="include the batched comparison")
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--batch-kicks", type=int, default=200)
    p.add_argument("--batch-seed", type=int, default=3)
    p.add_argument("--plain-sample", type=int, default=64,
                   help="batched: instances timed on the single-instance path")
    p.add_argument("--identity-sample", type=int, default=512,
                   help="batched: instances whose tours are checked against that path")
    p.add_argument("--serve-seconds", type=float, default=20.0,
                   help="serving block: seconds of Poisson arrivals (0 to skip)")
    p.add_argument("--serve-rate", type=float, default=2000.0)
    p.add_argument("--serve-drain", type=float, default=10.0)
    p.add_argument("--serve-rate-low", type=float, default=30.0,
                   help="serving: a second, sustainable arrival rate (0: skip)")
    return p.parse_args()


def workload(n, seed):
    xy = instances.clustered(n, seed, side=1.0e6, clusters=200, sigma_frac=0.01)
    route = lg.nn_tour(xy, 0)
    return xy, route


def pairs_per_sweep(n):
    return (n - 2) * (n - 3) // 2


def config(n, world):
    """The workload, identical for both arms (where a step runs is reported
    outside it, in `runs_on`)."""
    return {
        "workload": f"single large instance: n={n} Gaussian mixture (200 clusters, "
                    "sigma=1% of [0,1e6)^2, fp32), nearest-neighbour start tour, "
                    "best-improvement 2-opt descent moves",
        "n": n,
        "step": "one full sweep + argmin + move",
        "replicas": world,
    }


def cpu_model():
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for ln in r.stdout.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip() + f" ({platform.machine()})"
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model")):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


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
                 6: ("sweep_boxed_kernel", "boxed screen: near-neighbour seed bound, row-block "
                                           "and window bounding boxes, then the local-coordinate "
                                           "screen")}
# kernels per sweep launch: the boxed variant runs window_seed_kernel and tile_filter_kernel
# first
SWEEP_LAUNCHES = {6: 3}


def profile_figures(name):
    """`key: value` lines of the committed ncu summary profiles/<name>.md
    (figures taken from a capture of the command the file names), as floats;
    {} if the file is absent."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", f"{name}.md")) as f:
            for ln in f:
                if ln.startswith("bench_") and ":" in ln:
                    k, v = ln.split(":", 1)
                    try:
                        out[k.strip()[len("bench_"):]] = float(v.strip().split()[0])
                    except (ValueError, IndexError):
                        pass
    except OSError:
        pass
    return out


def lane_roofline(pairs, sweep_s, sm_mhz, prof):
    """Executed lane operations of a sweep over its live duration against the
    peak of 152 SMs x 128 FP32/INT32 lanes; beside it the pruning-inclusive
    convention figure (every pair charged 6 FP32 + 4 INT ops)."""
    peak = SMS * LANES * sm_mhz * 1e6
    conv = pairs / sweep_s * OPS_PER_PAIR
    out = {"peak": round(peak / 1e12, 3),
           "pairs_decided_per_s": pairs / sweep_s,
           "convention_frac": round(conv / peak, 4),
           "convention_note": "pairs decided x 10 ops / lane peak: counts pairs the box "
                              "tests rule out in blocks, so it measures pruning, not "
                              "lane throughput"}
    ti = prof.get("thread_inst_per_sweep")
    if ti:
        out["achieved"] = round(ti / sweep_s / 1e12, 3)
        out["frac"] = round(ti / sweep_s / peak, 4)
        out["lane_ops_per_sweep"] = ti
        out["lane_ops_per_pair"] = round(ti / pairs, 5)
    else:
        out["achieved"] = None
        out["frac"] = None
    if prof.get("issue_active_pct") is not None:
        out["issue_frac"] = round(prof["issue_active_pct"] / 100.0, 4)
    if prof.get("exact_pairs_per_sweep") is not None:
        out["pairs_exact"] = prof["exact_pairs_per_sweep"]
    out["traffic"] = prof.get("dram_bytes_per_sweep")
    return out


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
    """The largest v over the ranks (every rank gets it)."""
    if dist is None:
        return v
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, pairs, steps, seconds):
    """Whole-job throughput: every rank decides `pairs` pairs per step for
    `steps` steps (weak scaling), over the slowest rank's time."""
    return world * pairs * steps / seconds


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
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(a.steps)]
    barrier(dist)
    torch.cuda.synchronize()
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    time.sleep(0.4)
    t_wall = time.perf_counter()
    # the timed steps: events before the sweep and after the move only, so
    # nothing sits between the step's launches
    for k in range(a.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        ev[k][0].record(ext)
        s.enqueue_sweep()
        s.enqueue_apply()
        ev[k][1].record(ext)
    s.sync()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    barrier(dist)
    step_ms = [e[0].elapsed_time(e[1]) for e in ev]
    # the sweep alone (roofline of the dominant kernel): the next steps of
    # the same descent, with an event between the sweep and the move
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(a.steps)]
    for k in range(a.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        evs[k][0].record(ext)
        s.enqueue_sweep()
        evs[k][1].record(ext)
        s.enqueue_apply()
    s.sync()
    sweep_ms = [e[0].elapsed_time(e[1]) for e in evs]
    moves, converged = s.progress()
    if converged or moves != a.warmup + 2 * a.steps:
        raise RuntimeError(f"descent ended early ({moves} moves); pick fewer steps")
    total_s = reduce_max(dist, sum(step_ms) / 1e3)
    value = job_rate(world, pairs, a.steps, total_s)
    ms_per_step = total_s * 1e3 / a.steps

    # e2e: the C-ABI call with host buffers, one move per call
    cur = s.get_route()
    info_route_io = {lg.ROUTE_IO_COPY: "copy", lg.ROUTE_IO_DIRECT: "direct"}.get(
        s.info()["route_io"], "?")
    for _ in range(3):
        s.optimize_inplace(cur, max_moves=1)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        s.optimize_inplace(cur, max_moves=1)  # the caller's buffer, in and out
    e2e_s = reduce_max(dist, time.perf_counter() - t0)
    e2e = {"value": job_rate(world, pairs, a.e2e_steps, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n + 2 * 128,
           "call": "logo_descend(max_moves=1) per step on the caller's host buffer: "
                   "route in, sweep, argmin, reversal, route out (read and written in "
                   "place by the device where it reaches pageable host memory, else "
                   "copied)", "route_io": info_route_io}

    # roofline of the sweep (the dominant kernel: the boxed screen's three
    # launches, timed together by the events around logo_enqueue_sweep)
    info = s.info()
    kname, screen = SWEEP_KERNELS[info["variant"]]
    peaks = measured_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    mean_sweep_s = statistics.mean(sweep_ms) / 1e3
    prof_name = f"{kname}_n{n // 1000}k"
    roof = {"bound": "alu", "unit": "TOPS (lane operations)"}
    roof.update(lane_roofline(pairs, mean_sweep_s, sm_max, profile_figures(prof_name)))
    roof.update({
        "kernel": ("logo::window_seed_kernel + logo::tile_filter_kernel + "
                   if SWEEP_LAUNCHES.get(info["variant"]) else "")
                  + f"logo::{kname}<{info['rows_per_thread']},{info['warps_per_cta']}>"
                  + f" ({screen}, {info['tile_cols']}-column tiles; timed together)",
        "sweep_ms_mean": round(statistics.mean(sweep_ms), 4),
        "peak_source": f"152 SMs x 128 FP32/INT32 lanes x sm_max_mhz={sm_max:g} "
                       "(MEASURED_PEAKS.json)",
        "figures_source": f"profiles/{prof_name}.md: thread instructions, issue-slot use and "
                          "DRAM bytes per sweep from the ncu capture of this command's "
                          "timed sweeps; the duration is this run's",
    })
    if clocks.get("sm_mhz") and roof.get("lane_ops_per_sweep"):
        roof["frac_at_sampled_clock"] = round(
            roof["lane_ops_per_sweep"] / mean_sweep_s / (SMS * LANES * clocks["sm_mhz"] * 1e6), 4)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded Gaussian mixture, no dataset)",
        "config": config(n, world), "runs_on": "GPU" if world == 1 else f"{world} GPUs",
        "l2": "flushed between timed steps (256 MiB write); inputs 1.6 MB",
        "value_note": "pairs decided per second: all (n-2)(n-3)/2 pairs of each sweep, "
                      "whether evaluated one by one or ruled out with their block",
        "roofline": roof, "e2e": e2e, "clocks": clocks,
        "gpu_launches": (SWEEP_LAUNCHES.get(info["variant"], 1) + 1) * a.steps,
        "wall_s_timed_region": round(t_wall, 3),
    }

    def block(name, fn, *args):
        # an extra block that fails is reported in the line, not fatal to it
        try:
            out[name] = fn(*args)
        except Exception as e:  # noqa: BLE001
            out[name] = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0 and a.dense:
        block("dense", run_dense, s, xy, route, sm_max, local)
    if rank == 0 and a.sweep_sizes:
        block("sweep_per_n", run_sweep_per_n, a, sm_max, local)
    if rank == 0 and a.large_kicks:
        block("large", run_large, a, local)
    if a.batched and rank == 0:
        block("batched", run_batched, a, local)
    if a.serve_seconds > 0 and rank == 0:
        block("serving", run_serving, a, local)

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
            "cpu_model": cpu_model(),
            "same_move_as_gpu": oracle.unpack_key(key) == gpu_move,
        }
    s.close()
    return out


def _time_sweeps(s, reps, device):
    """CUDA-event time of `reps` sweeps of the resident tour (no move), L2
    flushed before each; returns the list of milliseconds."""
    import torch
    ext = torch.cuda.ExternalStream(s.stream, device=torch.device("cuda", device))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{device}")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    for e0, e1 in ev:
        s.begin_descent(0)
        with torch.cuda.stream(ext):
            flush.zero_()
        e0.record(ext)
        s.enqueue_sweep()
        e1.record(ext)
    s.sync()
    torch.cuda.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in ev]


def run_dense(s_main, xy, route, sm_max, device):
    """The local-coordinate screen (LOGO_SWEEP_LOCAL): every pair of the
    sweep is screened on its own (two FFMA per pair, exact distances where
    the screen passes), on the headline instance's start tour.  This is the
    kernel whose lane and issue use measure ALU efficiency; the boxed screen
    of the headline skips most of this work."""
    n = len(route)
    pairs = pairs_per_sweep(n)
    with lg.Solver(xy, device=device) as s:
        s.set_kernel(lg.SWEEP_LOCAL, 4, 4, 512)
        s.set_route(route)
        move = s.sweep_resident()
        ms = _time_sweeps(s, 8, device)
        info = s.info()
    s_main.set_route(route)
    same = s_main.sweep_resident() == move
    mean_s = statistics.mean(ms[1:]) / 1e3
    roof = {"bound": "alu", "unit": "TOPS (lane operations)"}
    roof.update(lane_roofline(pairs, mean_s, sm_max, profile_figures(f"sweep_kernel6_n{n // 1000}k")))
    return {"workload": f"one sweep of the headline instance's start tour (n={n}) with the "
                        "every-pair local-coordinate screen",
            "kernel": f"logo::sweep_kernel6<{info['rows_per_thread']},{info['warps_per_cta']},32> "
                      f"({info['tile_cols']}-column tiles)",
            "sweep_ms_mean": round(mean_s * 1e3, 4), "pair_evals_per_s": pairs / mean_s,
            "same_move_as_boxed": bool(same), "roofline": roof}


def run_sweep_per_n(a, sm_max, device):
    """One best-improvement sweep (no move) of uniform float32 points in
    [0,1e6)^2 on a random tour at each size; the default kernel per size."""
    rows = []
    for n in [int(x) for x in a.sweep_sizes.split(",") if x.strip()]:
        xy = instances.uniform_f32(n, 40 + n, 1.0e6)
        r = lg.random_tour(n, 41 + n)
        with lg.Solver(xy, device=device) as s:
            s.set_route(r)
            s.sweep_resident()
            ms = _time_sweeps(s, 3 if n >= 1000000 else 10, device)
            info = s.info()
        mean_s = statistics.mean(ms) / 1e3
        prof = profile_figures("sweep_per_n_uniform_random")
        key = f"n{n // 1000}k"
        sub = {k[len(key) + 1:]: v for k, v in prof.items() if k.startswith(key + "_")}
        row = {"n": n, "pairs": pairs_per_sweep(n), "sweep_ms": round(mean_s * 1e3, 4),
               "pair_evals_per_s": pairs_per_sweep(n) / mean_s, "variant": info["variant"],
               "shape": [info["rows_per_thread"], info["warps_per_cta"], info["tile_cols"]]}
        row.update(lane_roofline(pairs_per_sweep(n), mean_s, sm_max, sub))
        rows.append(row)
    return {"workload": "one sweep, uniform fp32 [0,1e6)^2, random tour, L2 flushed; "
                        "issue and lane figures from profiles/sweep_per_n_uniform_random.md",
            "results": rows}


def run_large(a, device):
    """The single large instance as a whole: descent from the
    nearest-neighbour tour, then `large_kicks` double-bridge ILS iterations
    (logo_ils, the ILS loop of ILSGlobalSolverSequential with a kick count)."""
    n = a.n
    xy, route = workload(n, a.seed)

    def one(search, k):
        with lg.Solver(xy, device=device) as s:
            s.set_search(search, k)
            s.ils(route[:], 2, 1, lg.KICK_DOUBLE_BRIDGE)  # warm-up (graphs, caches)
            t0 = time.perf_counter()
            tour, st = s.ils(route, a.large_kicks, a.seed, lg.KICK_DOUBLE_BRIDGE)
            wall = time.perf_counter() - t0
            t0 = time.perf_counter()
            _, dst = s.optimize(route)
            descent = time.perf_counter() - t0
        return {"wall_s": round(wall, 4), "device_s": round(st["device_ms"] / 1e3, 4),
                "pair_evals": st["pair_evals"],
                "pair_evals_per_s": st["pair_evals"] / (st["device_ms"] / 1e3),
                "moves": st["moves"], "sweeps": st["sweeps"], "accepted": st["accepted"],
                "start_length": st["start_length"], "final_length": st["final_length"],
                "valid_tour": bool(lg.check_tour(tour)),
                "descent_only_s": round(descent, 4), "descent_moves": dst["moves"],
                "descent_final_length": dst["final_length"]}

    out = {"workload": f"n={n} Gaussian mixture, NN start, descent + {a.large_kicks} "
                       "double-bridge kicks (logo_ils with host buffers)"}
    out.update(one(lg.SEARCH_EXHAUSTIVE, 0))
    # the same call with the neighbour-list search (8 nearest cities, then
    # full sweeps): another path to 2-opt local optima, not the reference's
    out["neighbour_search"] = one(lg.SEARCH_NEIGHBOUR, 8)
    # and with Or-opt moves among the neighbour candidates
    out["neighbour_oropt_search"] = one(lg.SEARCH_NEIGHBOUR_OROPT, 8)
    return out


def run_serving(a, device):
    """Poisson arrivals at `serve_rate`/s, n log-uniform in [100, 20000],
    clustered or uniform coordinates 50/50 by seed, NN start tours, each
    request a descent + 50 segment kicks; through logo_server (continuous
    batching) and, with the same arrival sequence, through the plain path
    (one request at a time on its own context)."""
    import bench_suite
    pool = bench_suite._pool(256, 5, 100, 20000)
    srv = bench_suite._serve_run(pool, a.serve_rate, a.serve_seconds, 50, a.serve_drain, 5)
    plain = bench_suite._plain_run(pool, a.serve_rate, a.serve_seconds, 50, a.serve_drain, 5)
    low = None
    if a.serve_rate_low > 0:
        # a rate the device sustains with this mix (the mean request needs
        # about 4e10 pair evaluations), where latency is service time
        # rather than queueing; the plain path beside it
        low = {"offered_per_s": a.serve_rate_low,
               "server": bench_suite._serve_run(pool, a.serve_rate_low, a.serve_seconds, 50,
                                                a.serve_drain, 6),
               "plain": bench_suite._plain_run(pool, a.serve_rate_low, a.serve_seconds, 50,
                                               a.serve_drain, 6)}
    return {"workload": f"Poisson arrivals at {a.serve_rate:g}/s for {a.serve_seconds:g} s "
                        "(+ drain), n log-uniform [100,20000], clustered/uniform 50/50, NN "
                        "start, descent + 50 kicks per request",
            "shortened": "the specified stream runs 600 s; the benchmark runs "
                         f"{a.serve_seconds:g} s of it so the whole run ends in minutes "
                         "(same rate and request mix)",
            "server": srv, "plain": plain,
            "completed_ratio": (srv["completed_per_s"] / plain["completed_per_s"]
                                if plain["completed_per_s"] else None),
            "sustainable": low}


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
    # plain: the single-instance path (logo_ils), one instance at a time, on a
    # stratified sample; context creation (allocations, tile list, graph
    # capture) is timed apart from the solves, and every sampled instance's
    # tour and length must equal the batched result
    isample = order[np.linspace(0, count - 1, min(count, a.identity_sample)).astype(int)]
    identical, setup_s, solve_s = 0, 0.0, 0.0
    for k in isample:
        t0 = time.perf_counter()
        s = lg.Solver(coords[k], device=device)
        t1 = time.perf_counter()
        r, st = s.ils(routes[k], kicks, seeds[k], lg.KICK_SEGMENT)
        t2 = time.perf_counter()
        s.close()
        setup_s += t1 - t0
        solve_s += t2 - t1
        identical += int(st["final_length"] == res[k]["best_length"] and
                         np.array_equal(r, got[k]))
    plain = len(isample) * (kicks + 1) / solve_s
    lengths_ok = all(r["status"] == 0 for r in res)
    return {
        "workload": f"{count} instances, n log-uniform in [50,2000], uniform fp32 in "
                    f"[0,1e4)^2, random start, descent + {kicks} segment kicks each",
        "metric": "local-opts/s", "value": batched, "device_s": ms / 1e3,
        "pair_evals_per_s": float((sweeps * pairs).sum() / (ms / 1e3)),
        "moves": int(sum(r["moves"] for r in res)),
        "plain": {"value": plain, "unit": "local-opts/s", "sample": int(len(isample)),
                  "solve_s": solve_s, "context_setup_s": setup_s,
                  "how": "logo_ils per instance on its own context, stratified by n; "
                         "context creation timed separately"},
        "speedup_vs_plain": batched / plain,
        "identical_tours_and_lengths": f"{identical}/{len(isample)}",
        "all_statuses_ok": bool(lengths_ok),
        "autotuned_shapes": shapes, "autotune_s": tune_s,
    }


def run_reference(a, rank):
    """The reference CPU path on the host cores: the oracle port of
    CPUMTSolver::optimizeStep (src/solvers/cpuMTSolver.cpp:31-158) + the move
    application (src/solvers/twoOptLocalSolver.cpp:41-48) on all threads, on
    the same instance, start tour, warm-up and step count as our arm."""
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
    for _ in range(a.warmup):
        r = step(r)
    steps = a.steps
    t0 = time.perf_counter()
    done = 0
    for _ in range(steps):
        r = step(r)
        done += 1
        # a very long request (thousands of steps) is cut at 10 minutes of CPU work
        if time.perf_counter() - t0 > 600.0:
            break
    el = time.perf_counter() - t0
    value = pairs * done / el
    sample = (f"{done} descent steps (full {n}-city sweep + move) of the benchmark "
              f"workload after {a.warmup} warm-up steps, on {threads} threads")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": done, "warmup": a.warmup, "ms_per_step": el * 1e3 / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Gaussian mixture, no dataset)",
        "config": config(n, 1), "runs_on": "host cores",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(), "sample": sample},
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
