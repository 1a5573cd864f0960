"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Every expected value here comes from oracle/_ref/ref_harness, which runs the
reference's unmodified C++ sources (TwoOptLocalSolver::optimize, routeLength,
ILSGlobalSolver::kick, ILSGlobalSolverSequential::optimize, initRoute_KD_NN,
multipleFragment_KD, readFileCoords) with the per-edge nint optimizeStep -- see oracle/build_ref.sh.
Instances are regenerated from (generator, n, seed) by instances.py; each
fixture stores a SHA-256 of the instance and start tour so a drift of the
generators is caught before any comparison.

Run (x86-64 host with the reference checkout):
    python tests/golden/make_golden.py [--ref /root/reference]
"""
import argparse
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "logo-tsp-solver_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import instances  # noqa: E402
import ref  # noqa: E402

GENS = ["uniform_int", "uniform_f32", "clustered"]
TSPLIB = ["berlin52", "kroA100", "pr2392"]


def make_instance(gen, n, seed):
    if gen == "uniform_int":
        return instances.uniform_int(n, seed)
    if gen == "uniform_f32":
        return instances.uniform_f32(n, seed, 1.0e4)
    return instances.clustered(n, seed, side=1.0e6, clusters=max(2, n // 50))


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def steps():
    rows, outs, hashes = [], [], []
    sizes = [5, 6, 7, 8, 10, 16, 33, 64, 100, 200, 500, 1000, 2000, 5000]
    for n in sizes:
        per = 12 if n <= 100 else (6 if n <= 1000 else 2)
        for gi, gen in enumerate(GENS):
            for s in range(per):
                seed = 1000 * n + 10 * gi + s
                xy = make_instance(gen, n, seed)
                r = instances.random_tour(n, seed + 1)
                outs.append(ref.step(xy, r))
                rows.append((gi, n, seed, seed + 1))
                hashes.append(digest(xy, r))
    return {"spec": np.array(rows, dtype=np.int64), "out": np.array(outs, dtype=np.int32),
            "hash": np.array(hashes)}


def small_n():
    """Tours of 4 to 7 cities: single steps and whole descents.  At n = 4 the
    reference's loop (src/solvers/cpuSolver.cpp:104,123: i < n-2, j < n-1)
    evaluates exactly one pair, (i, j) = (1, 2), reported as (1, 3)."""
    rows, outs, hashes, logs, fin = [], [], [], [], []
    square = np.array([[0, 0], [10, 0], [10, 10], [0, 10]], dtype=np.float32)
    cases = [("square", square, np.array([0, 2, 1, 3], dtype=np.uint32), -1, -1)]
    for n in (4, 5, 6, 7):
        for gi, gen in enumerate(GENS):
            for s in range(8):
                seed = 7000 * n + 10 * gi + s
                cases.append((gen, make_instance(gen, n, seed),
                              instances.random_tour(n, seed + 1), seed, gi))
    for gen, xy, r, seed, gi in cases:
        n = len(r)
        outs.append(ref.step(xy, r))
        fr, m, log, length = ref.descend(xy, r)
        logs.append(log)
        rows.append((gi, n, seed, seed + 1, m, length))
        hashes.append(digest(xy, r))
        fin.append(fr)
    off = np.cumsum([0] + [len(x) for x in logs]).astype(np.int64)
    foff = np.cumsum([0] + [len(x) for x in fin]).astype(np.int64)
    return {"spec": np.array(rows, dtype=np.int64), "out": np.array(outs, dtype=np.int32),
            "hash": np.array(hashes), "log": np.concatenate(logs).reshape(-1, 3).astype(np.int32),
            "log_offsets": off, "final": np.concatenate(fin).astype(np.uint32),
            "final_offsets": foff}


def descents():
    logs, meta, hashes, fin = [], [], [], []
    for seed in range(1, 17):
        xy = instances.uniform_int(1000, seed)
        r = instances.random_tour(1000, seed)
        fr, m, log, length = ref.descend(xy, r)
        logs.append(log)
        meta.append((seed, m, length))
        hashes.append(digest(xy, r))
        fin.append(digest(fr))
    off = np.cumsum([0] + [len(x) for x in logs]).astype(np.int64)
    return {"log": np.concatenate(logs).astype(np.int32), "offsets": off,
            "meta": np.array(meta, dtype=np.int64), "hash": np.array(hashes),
            "final_hash": np.array(fin)}


def kicks_and_ils():
    krows, khash, kout, kstate = [], [], [], []
    for n in (5, 9, 50, 333, 2000):
        for s in range(4):
            seed = 77 * n + s
            xy = instances.uniform_int(n, seed)
            r = instances.random_tour(n, seed)
            rk, st = ref.kick(xy, r, seed * 31 + 7, 5)
            krows.append((n, seed, seed * 31 + 7, 5))
            khash.append(digest(xy, r))
            kout.append(digest(rk))
            kstate.append(st)
    irows, ihash, iout = [], [], []
    for n, kicks in ((60, 30), (200, 20), (300, 12)):
        for s in range(2):
            seed = 5 * n + s
            xy = instances.uniform_f32(n, seed, 1.0e4)
            r = instances.random_tour(n, seed)
            br, bl, moves = ref.ils(xy, r, kicks, seed + 99)
            irows.append((n, seed, kicks, seed + 99, bl, moves))
            ihash.append(digest(xy, r))
            iout.append(digest(br))
    return {"kick_spec": np.array(krows, dtype=np.uint64), "kick_hash": np.array(khash),
            "kick_out": np.array(kout), "kick_state": np.array(kstate, dtype=np.uint64),
            "ils_spec": np.array(irows, dtype=np.int64), "ils_hash": np.array(ihash),
            "ils_out": np.array(iout)}


def nn_tours():
    rows, h, out = [], [], []
    for gen, n, seed in (("clustered", 5000, 3), ("uniform_f32", 2000, 5),
                         ("uniform_int", 1000, 1), ("clustered", 20000, 8)):
        xy = make_instance(gen, n, seed)
        t = ref.nn_tour(xy)
        rows.append((GENS.index(gen), n, seed))
        h.append(digest(xy))
        out.append(digest(t))
    return {"spec": np.array(rows, dtype=np.int64), "hash": np.array(h), "out": np.array(out)}


def mf_tours(refdir):
    """Multiple-fragment start tours (multipleFragment_KD) on seeded instances
    and TSPLIB files whose neighbour searches have no exact distance ties."""
    rows, h, out = [], [], []
    for gen, sizes in (("uniform_f32", (3, 4, 5, 7, 10, 31, 100, 500, 2000, 10000)),
                       ("clustered", (5, 10, 100, 500, 2000, 10000)),
                       ("uniform_int", (4, 6, 10, 100, 500, 2000))):
        for n in sizes:
            for seed in (1, 2):
                xy = make_instance(gen, n, seed)
                rows.append((GENS.index(gen), n, seed))
                h.append(digest(xy))
                out.append(digest(ref.mf_tour(xy)))
    d = {"spec": np.array(rows, dtype=np.int64), "hash": np.array(h), "out": np.array(out)}
    for name in ("berlin52", "kroA100", "att532"):
        xy = ref.read_tsp(os.path.join(refdir, "TSPLIB", name + ".tsp"))
        d[name + "_xy"] = xy
        d[name + "_mf"] = ref.mf_tour(xy)
    return d


def tsplib(refdir):
    d = {}
    for name in TSPLIB:
        xy = ref.read_tsp(os.path.join(refdir, "TSPLIB", name + ".tsp"))
        nn = ref.nn_tour(xy)
        fr, m, log, length = ref.descend(xy, nn) if len(xy) <= 200 else (None, 0, None, 0)
        d[name + "_xy"] = xy
        d[name + "_nn"] = nn
        d[name + "_step"] = np.array(ref.step(xy, nn), dtype=np.int32)
        if fr is not None:
            d[name + "_log"] = log
            d[name + "_final"] = fr
            d[name + "_len"] = np.array([length, ref.length(xy, nn)], dtype=np.int64)
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default=None, help="write only this fixture (e.g. mf_tours)")
    a = ap.parse_args()
    if not ref.available():
        ref.build()
    if a.only == "mf_tours":
        np.savez_compressed(os.path.join(HERE, "mf_tours.npz"), **mf_tours(a.ref))
        print("mf_tours.npz written to", HERE)
        return
    if a.only == "small_n":
        np.savez_compressed(os.path.join(HERE, "small_n.npz"), **small_n())
        print("small_n.npz written to", HERE)
        return
    np.savez_compressed(os.path.join(HERE, "small_n.npz"), **small_n())
    np.savez_compressed(os.path.join(HERE, "mf_tours.npz"), **mf_tours(a.ref))
    np.savez_compressed(os.path.join(HERE, "steps.npz"), **steps())
    np.savez_compressed(os.path.join(HERE, "descents_n1000.npz"), **descents())
    np.savez_compressed(os.path.join(HERE, "kicks_ils.npz"), **kicks_and_ils())
    np.savez_compressed(os.path.join(HERE, "nn_tours.npz"), **nn_tours())
    np.savez_compressed(os.path.join(HERE, "tsplib.npz"), **tsplib(a.ref))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
