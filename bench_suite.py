"""Benchmarks of the workloads beside bench.py's headline (one JSON line each).

  python bench_suite.py plain    # n=1000 integer coords, descent
  python bench_suite.py sweep    # one sweep at n=10k, 100k, 1M
  python bench_suite.py large    # n=100k NN descent + 1000 kicks
  python bench_suite.py serve    # Poisson request stream
  python bench_suite.py construct  # start tours, host vs device

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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "logo-tsp-solver_gb300"))

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
            info = s.info()
            if a.reps == 0:  # one sweep per size (for profiling): no timing
                out.append({"n": n, "variant": info["variant"], "move": list(move)})
                continue
            ts = _time_sweeps(s, a.reps or (3 if n >= 1000000 else 12))
            best = min(ts[1:]) if len(ts) > 1 else ts[0]
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


def cmd_construct(a):
    """Start tours for the batched workload (4096 instances, n log-uniform in
    [50, 2000], uniform fp32 in [0,1e4)^2): nearest-neighbour tours built on
    the host (logo_nn_tour, one instance after another) and then solved, vs
    built by the batched launch itself (start=START_NN); both then descend to
    a local optimum.  The same for multiple-fragment tours (logo_mf_tour on
    the host vs start=START_MF, built by a launch before the solve)."""
    coords, _, seeds = instances.batched_workload(a.count, a.seed, 50, 2000, 1.0e4)
    total = sum(len(c) for c in coords)
    t0 = time.perf_counter()
    nn = [lg.nn_tour(c, 0) for c in coords]
    host_nn_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    mf = [lg.mf_tour(c) for c in coords]
    host_mf_s = time.perf_counter() - t0
    with lg.Batch(len(coords), total) as b:
        b.solve(coords[:64], nn[:64], seeds[:64])  # warm-up
        t0 = time.perf_counter()
        r_given, res_given, ms_given = b.solve(coords, nn, seeds)
        given_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        r_dev, res_dev, ms_dev = b.solve(coords, None, seeds, start=lg.START_NN)
        dev_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        r_mfg, _, ms_mfg = b.solve(coords, mf, seeds)
        mf_given_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        r_mfd, _, ms_mfd = b.solve(coords, None, seeds, start=lg.START_MF)
        mf_dev_s = time.perf_counter() - t0
    same = all(np.array_equal(x, y) for x, y in zip(r_given, r_dev))
    same_mf = all(np.array_equal(x, y) for x, y in zip(r_mfg, r_mfd))
    print(json.dumps({"workload": f"construct: {a.count} instances, n log-uniform [50,2000], "
                                  "NN start tours, descent to a local optimum",
                      "host_nn_s": host_nn_s, "host_mf_s": host_mf_s,
                      "solve_given_nn_device_ms": ms_given, "solve_given_nn_wall_s": given_s,
                      "solve_device_nn_device_ms": ms_dev, "solve_device_nn_wall_s": dev_s,
                      "device_construction_ms": ms_dev - ms_given,
                      "end_to_end_host_nn_s": host_nn_s + given_s,
                      "end_to_end_device_nn_s": dev_s, "identical_results": same,
                      "solve_given_mf_device_ms": ms_mfg, "solve_device_mf_device_ms": ms_mfd,
                      "device_mf_construction_ms": ms_mfd - ms_mfg,
                      "end_to_end_host_mf_s": host_mf_s + mf_given_s,
                      "end_to_end_device_mf_s": mf_dev_s, "identical_results_mf": same_mf}))


def cmd_search(a):
    """Descent of bench.py's instance (n = --n, Gaussian mixture, NN start)
    with the neighbour-list search (--k nearest cities), limited to --limit
    moves (0: to the local optimum), beside the exhaustive search."""
    import bench
    xy, r0 = bench.workload(a.n, a.seed)
    res = []
    for search, k in ((lg.SEARCH_NEIGHBOUR, a.k), (lg.SEARCH_EXHAUSTIVE, 0)):
        if search == lg.SEARCH_EXHAUSTIVE and a.limit:
            continue  # profiling runs: the neighbour search alone
        with lg.Solver(xy) as s:
            s.set_search(search, k)
            t0 = time.perf_counter()
            got, st = s.optimize(r0, max_moves=a.limit)
            wall = time.perf_counter() - t0
        res.append({"search": "neighbour" if search else "exhaustive", "k": k,
                    "wall_s": wall, "moves": st["moves"], "sweeps": st["sweeps"],
                    "final_length": st["final_length"], "pair_evals": st["pair_evals"]})
    print(json.dumps({"workload": f"n={a.n} Gaussian mixture, NN start, descent"
                                  + (f" limited to {a.limit} moves" if a.limit else ""),
                      "results": res}))


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


def _serve_run(pool, rate, duration, kicks, drain, seed, max_large=0):
    """Poisson arrivals through logo_server.  A collector thread polls every
    outstanding request, so a long request does not hide later completions;
    latencies are the server's own (submit to result)."""
    rng = np.random.default_rng(seed)
    t_arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 1.2) + 10))
    t_arr = t_arr[t_arr < duration]
    picks = rng.integers(0, len(pool), size=len(t_arr))
    done = {}
    outstanding = set()
    lock = threading.Lock()
    stop = threading.Event()
    with lg.Server(kicks=kicks, kind=lg.KICK_SEGMENT, max_large=max_large) as srv:
        t0 = time.perf_counter()

        def collect():
            while True:
                last = stop.is_set()
                with lock:
                    cur = list(outstanding)
                for rid in cur:
                    res = srv.poll(rid)
                    if res is not None:
                        done[rid] = (res[1], time.perf_counter() - t0)
                        with lock:
                            outstanding.discard(rid)
                if last:
                    return
                time.sleep(0.01)

        th = threading.Thread(target=collect, daemon=True)
        th.start()
        n_sub = 0
        for t, p in zip(t_arr, picks):
            now = time.perf_counter() - t0
            if t > now:
                time.sleep(t - now)
            xy, r, s = pool[p]
            rid = srv.submit(xy, r, s)
            with lock:
                outstanding.add(rid)
            n_sub += 1
        sub_end = time.perf_counter() - t0
        while time.perf_counter() - t0 < duration + drain:
            with lock:
                if not outstanding:
                    break
            time.sleep(0.05)
        stop.set()
        th.join()
        st = srv.stats()
        wall = time.perf_counter() - t0
    infos = [d for d, _ in done.values() if "error" not in d]
    lat = [d["latency_ms"] for d in infos]
    work = sum(d["sweeps"] * pairs(d["n"]) for d in infos)
    return {"offered_per_s": rate, "duration_s": duration, "submitted": n_sub,
            "completed": len(infos), "completed_per_s": len(infos) / wall, "wall_s": wall,
            "submit_s": sub_end, "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
            "queue_p50_ms": _pct([d["queue_ms"] for d in infos], 50),
            "pair_evals_per_s": work / wall, "failed": len(done) - len(infos),
            "pending_at_end": st["pending"], "rounds": st["rounds"],
            "round_device_s": st["round_device_ms"] / 1e3}


def _characterize(pool, kicks):
    """Each pool instance once through logo_ils: the work a request needs
    (pair evaluations) and its one-at-a-time device time."""
    rows = []
    for xy, r, s in pool:
        with lg.Solver(xy) as sol:
            _, st = sol.ils(r, kicks, s, lg.KICK_SEGMENT)
        rows.append((len(r), st["pair_evals"], st["device_ms"]))
    n = np.array([x[0] for x in rows])
    w = np.array([x[1] for x in rows], dtype=np.float64)
    ms = np.array([x[2] for x in rows])
    big = n > 4096
    return {"instances": len(rows), "mean_pair_evals": float(w.mean()),
            "work_share_above_4096": float(w[big].sum() / w.sum()),
            "share_above_4096": float(big.mean()),
            "mean_device_ms_one_at_a_time": float(ms.mean()),
            "req_per_s_bound_at_7e12": 7.0e12 / float(w.mean())}


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
    if a.characterize:
        res.append({"characterize": _characterize(pool, a.kicks)})
    for rate in rates:
        srv = _serve_run(pool, rate, a.duration, a.kicks, a.drain, a.seed, a.max_large)
        plain = (_plain_run(pool, rate, a.duration, a.kicks, a.drain, a.seed)
                 if a.plain else None)
        res.append({"rate": rate, "max_large": a.max_large, "server": srv, "plain": plain})
    print(json.dumps({"workload": f"serving: Poisson arrivals, n log-uniform "
                                  f"[{a.n_lo},{a.n_hi}], clustered/uniform 50/50, NN start, "
                                  f"descent + {a.kicks} kicks",
                      "pool": a.pool, "results": res}))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("cmd", choices=["plain", "sweep", "large", "serve", "construct", "search"])
    p.add_argument("--n", type=int, default=100000, help="search: cities")
    p.add_argument("--k", type=int, default=8, help="search: neighbour-list length")
    p.add_argument("--limit", type=int, default=0, help="search: move limit (0: none)")
    p.add_argument("--seeds", type=int, default=4)
    p.add_argument("--count", type=int, default=4096, help="construct: instances")
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--kicks", type=int, default=None)
    p.add_argument("--rates", default="2000,40")
    p.add_argument("--duration", type=float, default=10.0)
    p.add_argument("--drain", type=float, default=10.0)
    p.add_argument("--pool", type=int, default=256)
    p.add_argument("--n-lo", type=int, default=100)
    p.add_argument("--n-hi", type=int, default=20000)
    p.add_argument("--sizes", default="10000,100000,1000000")
    p.add_argument("--reps", type=int, default=None,
                   help="sweep: timed sweeps per size (0: one untimed sweep, for profiling)")
    p.add_argument("--max-large", type=int, default=0,
                   help="serve: requests above the batch limit in flight (0 = default)")
    p.add_argument("--plain", type=int, default=1, help="serve: also time the plain path")
    p.add_argument("--characterize", type=int, default=0,
                   help="serve: first run every pool instance once and report its work")
    a = p.parse_args()
    if a.kicks is None:
        a.kicks = {"large": 1000, "serve": 50}.get(a.cmd, 0)
    lg.load()
    {"plain": cmd_plain, "sweep": cmd_sweep, "large": cmd_large, "serve": cmd_serve,
     "construct": cmd_construct, "search": cmd_search}[a.cmd](a)


if __name__ == "__main__":
    main()
