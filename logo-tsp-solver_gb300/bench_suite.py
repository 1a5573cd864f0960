"""Benchmarks of the workloads beside bench.py's headline (one JSON line each).

  python logo-tsp-solver_gb300/bench_suite.py plain    # n=1000 integer coords, descent
  python logo-tsp-solver_gb300/bench_suite.py sweep    # one sweep at n=10k, 100k, 1M
  python logo-tsp-solver_gb300/bench_suite.py large    # n=100k NN descent + 1000 kicks
  python logo-tsp-solver_gb300/bench_suite.py serve    # Poisson request stream

All inputs are seeded synthetic instances (instances.py).  The oracle (CPU
restatement of the reference) is used only where a line reports a CPU
baseline or a parity check.
"""
import argparse
import json
import os
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)

import instances  # noqa: E402
import logo_gpu as lg  # noqa: E402

SMS, LANES, OPS_PER_PAIR = 152, 128, 10


def pairs(n):
    return (n - 2) * (n - 3) // 2


def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as o
    return o


def peak_ops():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f).get("sm_max_mhz", 2070.0))
    except (OSError, ValueError):
        mhz = 2070.0
    return SMS * LANES * mhz * 1e6


def cmd_plain(a):
    """n=1000 integer coordinates in [0,1e4)^2, random start, best-improvement
    descent to a local optimum; move sequence checked against the oracle."""
    o = oracle()
    rows = []
    for seed in range(1, a.seeds + 1):
        xy = instances.uniform_int(1000, seed)
        r = instances.random_tour(1000, seed)
        with lg.Solver(xy) as s:
            s.optimize(r)  # warm-up
            t0 = time.perf_counter()
            got, trace, st = s.optimize_trace(r)
            wall = time.perf_counter() - t0
        t0 = time.perf_counter()
        want, m, log = o.descend(xy, r, log_cap=1 << 20)
        cpu = time.perf_counter() - t0
        rows.append({"seed": seed, "moves": st["moves"], "final_length": st["final_length"],
                     "gpu_ms": st["device_ms"], "wall_ms": wall * 1e3, "cpu_oracle_ms": cpu * 1e3,
                     "identical_move_sequence": bool(np.array_equal(trace, log)),
                     "identical_tour": bool(np.array_equal(got, want))})
    ms = np.array([x["gpu_ms"] for x in rows])
    print(json.dumps({"workload": "plain: n=1000 integer coords [0,1e4)^2, random start, descent",
                      "descents_per_s": float(1e3 / ms.mean()), "gpu_ms_mean": float(ms.mean()),
                      "pair_evals_per_s": float(np.mean([(x["moves"] + 1) * pairs(1000) /
                                                         (x["gpu_ms"] / 1e3) for x in rows])),
                      "cpu_oracle_ms_mean": float(np.mean([x["cpu_oracle_ms"] for x in rows])),
                      "all_identical": all(x["identical_move_sequence"] and x["identical_tour"]
                                           for x in rows), "runs": rows}))


def _time_sweeps(s, reps):
    import torch
    ext = torch.cuda.ExternalStream(s.stream)
    ts = []
    for _ in range(reps):
        s.begin_descent(0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.enqueue_sweep()
        e1.record(ext)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return ts


def cmd_sweep(a):
    """One best-improvement sweep (no reversal) at n = 10k, 100k, 1M on uniform
    float32 points in [0,1e6)^2 and a random tour."""
    peak = peak_ops()
    out = []
    for n in [int(x) for x in a.sizes.split(",")]:
        xy = instances.uniform_f32(n, 40 + n, 1.0e6)
        r = lg.random_tour(n, 41 + n)
        with lg.Solver(xy) as s:
            s.set_route(r)
            move = s.sweep_resident()
            ts = _time_sweeps(s, 3 if n >= 1000000 else 12)
            best = min(ts[1:])
            info = s.info()
        ps = pairs(n) / (best / 1e3)
        out.append({"n": n, "pairs": pairs(n), "sweep_ms": best, "pair_evals_per_s": ps,
                    "alu_frac": ps * OPS_PER_PAIR / peak, "variant": info["variant"],
                    "shape": [info["rows_per_thread"], info["warps_per_cta"], info["tile_cols"]],
                    "move": list(move)})
    print(json.dumps({"workload": "sweep: one sweep, uniform fp32 [0,1e6)^2, random tour",
                      "peak_tops": peak / 1e12, "results": out}))


def cmd_large(a):
    """n=100,000 Gaussian mixture, NN start, full descent then `kicks`
    double-bridge ILS iterations."""
    n = 100000
    xy = instances.clustered(n, a.seed, side=1.0e6, clusters=200, sigma_frac=0.01)
    r = lg.nn_tour(xy, 0)
    with lg.Solver(xy) as s:
        t0 = time.perf_counter()
        tour, st = s.ils(r, a.kicks, a.seed, lg.KICK_DOUBLE_BRIDGE)
        wall = time.perf_counter() - t0
    print(json.dumps({"workload": f"large: n={n} Gaussian mixture, NN start, descent + "
                                  f"{a.kicks} double-bridge kicks",
                      "wall_s": wall, "device_s": st["device_ms"] / 1e3,
                      "pair_evals": st["pair_evals"],
                      "pair_evals_per_s": st["pair_evals"] / (st["device_ms"] / 1e3),
                      "alu_frac": st["pair_evals"] / (st["device_ms"] / 1e3) * OPS_PER_PAIR /
                      peak_ops(),
                      "moves": st["moves"], "sweeps": st["sweeps"], "accepted": st["accepted"],
                      "start_length": st["start_length"], "final_length": st["final_length"],
                      "valid_tour": lg.check_tour(tour)}))


def _pool(count, seed, n_lo, n_hi):
    """Serving instances: n log-uniform in [n_lo, n_hi], clustered or uniform
    (50/50 by seed) in [0,1e6)^2, nearest-neighbour start tours."""
    ns = instances.batch_sizes(count, seed, n_lo, n_hi)
    pool = []
    for k, n in enumerate(ns):
        s = instances.instance_seed(seed, k)
        n = int(n)
        if s & 1:
            xy = instances.clustered(n, s, side=1.0e6, clusters=max(2, n // 500))
        else:
            xy = instances.uniform_f32(n, s, 1.0e6)
        pool.append((xy, lg.nn_tour(xy, 0), s))
    return pool


def _pct(v, q):
    return float(np.percentile(v, q)) if len(v) else None


def _serve_run(pool, rate, duration, kicks, drain, seed):
    rng = np.random.default_rng(seed)
    t_arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 1.2) + 10))
    t_arr = t_arr[t_arr < duration]
    picks = rng.integers(0, len(pool), size=len(t_arr))
    lat, qms, done_at = [], [], []
    with lg.Server(kicks=kicks, kind=lg.KICK_SEGMENT) as srv:
        ids = []
        t0 = time.perf_counter()
        for t, p in zip(t_arr, picks):
            now = time.perf_counter() - t0
            if t > now:
                time.sleep(t - now)
            xy, r, s = pool[p]
            ids.append(srv.submit(xy, r, s))
        sub_end = time.perf_counter() - t0
        deadline = t0 + duration + drain
        for rid in ids:
            left = deadline - time.perf_counter()
            if left <= 0:
                break
            res = srv.wait(rid, int(left * 1e3))
            if res is None:
                break
            _, info = res
            lat.append(info["latency_ms"])
            qms.append(info["queue_ms"])
        st = srv.stats()
        wall = time.perf_counter() - t0
    return {"offered_per_s": rate, "duration_s": duration, "submitted": len(ids),
            "completed": len(lat), "completed_per_s": len(lat) / wall, "wall_s": wall,
            "submit_s": sub_end, "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
            "queue_p50_ms": _pct(qms, 50), "pending_at_end": st["pending"],
            "rounds": st["rounds"], "round_device_s": st["round_device_ms"] / 1e3}


def _plain_run(pool, rate, duration, kicks, drain, seed):
    """The same arrival sequence through the plain path: one request at a time
    (logo_ils on its own context), first come first served."""
    rng = np.random.default_rng(seed)
    t_arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 1.2) + 10))
    t_arr = t_arr[t_arr < duration]
    picks = rng.integers(0, len(pool), size=len(t_arr))
    lat = []
    t0 = time.perf_counter()
    for t, p in zip(t_arr, picks):
        now = time.perf_counter() - t0
        if now > duration + drain:
            break
        if t > now:
            time.sleep(t - now)
        xy, r, s = pool[p]
        with lg.Solver(xy) as sol:
            sol.ils(r, kicks, s, lg.KICK_SEGMENT)
        lat.append((time.perf_counter() - t0 - t) * 1e3)
    wall = time.perf_counter() - t0
    return {"offered_per_s": rate, "submitted": len(t_arr), "completed": len(lat),
            "completed_per_s": len(lat) / wall, "p50_ms": _pct(lat, 50),
            "p99_ms": _pct(lat, 99), "wall_s": wall}


def cmd_serve(a):
    pool = _pool(a.pool, a.seed, a.n_lo, a.n_hi)
    rates = [float(x) for x in a.rates.split(",")]
    res = []
    for rate in rates:
        srv = _serve_run(pool, rate, a.duration, a.kicks, a.drain, a.seed)
        plain = _plain_run(pool, rate, a.duration, a.kicks, a.drain, a.seed)
        res.append({"rate": rate, "server": srv, "plain": plain})
    print(json.dumps({"workload": f"serving: Poisson arrivals, n log-uniform "
                                  f"[{a.n_lo},{a.n_hi}], clustered/uniform 50/50, NN start, "
                                  f"descent + {a.kicks} kicks",
                      "pool": a.pool, "results": res}))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("cmd", choices=["plain", "sweep", "large", "serve"])
    p.add_argument("--seeds", type=int, default=4)
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--kicks", type=int, default=None)
    p.add_argument("--rates", default="2000,40")
    p.add_argument("--duration", type=float, default=10.0)
    p.add_argument("--drain", type=float, default=10.0)
    p.add_argument("--pool", type=int, default=256)
    p.add_argument("--n-lo", type=int, default=100)
    p.add_argument("--n-hi", type=int, default=20000)
    p.add_argument("--sizes", default="10000,100000,1000000")
    a = p.parse_args()
    if a.kicks is None:
        a.kicks = {"large": 1000, "serve": 50}.get(a.cmd, 0)
    lg.load()
    {"plain": cmd_plain, "sweep": cmd_sweep, "large": cmd_large, "serve": cmd_serve}[a.cmd](a)


if __name__ == "__main__":
    main()
