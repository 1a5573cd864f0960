"""Runs the reference's own code for the 2-opt path through
oracle/_ref/ref_harness (built by oracle/build_ref.sh from the reference
checkout) -- TEST INFRASTRUCTURE ONLY, used to pin the oracle.

Each call runs the harness in a fresh process: the reference keeps its
kd-tree and ILS history in static objects (src/utils/kdtree_utils.c:27,
src/solvers/ILSGlobalSolver.h:201-202) that only a new process resets.
"""
import os
import struct
import subprocess
import tempfile

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(_HERE, "_ref", "ref_harness")


def available():
    return os.path.exists(HARNESS)


def build():
    subprocess.run([os.path.join(_HERE, "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    return available()


def _run(cmd, xy, route, *extra):
    xy = np.ascontiguousarray(xy, dtype=np.float32).reshape(-1)
    route = np.ascontiguousarray(route, dtype=np.uint32)
    n = len(route)
    with tempfile.TemporaryDirectory() as d:
        fin = os.path.join(d, "in.bin")
        fout = os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<I", n))
            f.write(xy[: 2 * n].tobytes())
            f.write(route.tobytes())
        subprocess.run([HARNESS, cmd, fin, fout] + [str(e) for e in extra], check=True,
                       stdout=subprocess.DEVNULL)
        with open(fout, "rb") as f:
            return f.read()


def _route(buf, off):
    (n,) = struct.unpack_from("<I", buf, off)
    r = np.frombuffer(buf, dtype=np.uint32, count=n, offset=off + 4).copy()
    return r, off + 4 + 4 * n


def descend(xy, route):
    """TwoOptLocalSolver::optimize with per-edge nint steps.
    Returns (final_route, moves, log (m,3), final_length)."""
    b = _run("descend", xy, route)
    (m,) = struct.unpack_from("<Q", b, 0)
    log = np.frombuffer(b, dtype=np.int32, count=3 * m, offset=8).reshape(m, 3).copy()
    r, off = _route(b, 8 + 12 * m)
    (length,) = struct.unpack_from("<Q", b, off)
    return r, m, log, length


def avx_step(xy, route):
    """CPUSolver::optimizeStep as shipped (AVX, approximate sqrt)."""
    b = _run("avxstep", xy, route)
    return struct.unpack_from("<iii", b, 0)


def length(xy, route):
    return struct.unpack_from("<Q", _run("length", xy, route), 0)[0]


def kick(xy, route, seed, count=1):
    """ILSGlobalSolver::kick applied `count` times. Returns (route, rng_state)."""
    b = _run("kick", xy, route, seed, count)
    r, off = _route(b, 0)
    return r, struct.unpack_from("<Q", b, off)[0]


def ils(xy, route, kicks, seed):
    """ILSGlobalSolverSequential::optimize for `kicks` kicks.
    Returns (best_route, best_length, moves)."""
    b = _run("ils", xy, route, kicks, seed)
    (length,) = struct.unpack_from("<Q", b, 0)
    r, off = _route(b, 8)
    (moves,) = struct.unpack_from("<Q", b, off)
    return r, length, moves


def nn_tour(xy):
    n = len(np.asarray(xy).reshape(-1)) // 2
    b = _run("nn", xy, np.arange(n, dtype=np.uint32))
    return _route(b, 0)[0]


def mf_tour(xy):
    """The reference's multiple-fragment start tour (multipleFragment_KD)."""
    n = len(np.asarray(xy).reshape(-1)) // 2
    b = _run("mf", xy, np.arange(n, dtype=np.uint32))
    return _route(b, 0)[0]


def read_tsp(path):
    with tempfile.TemporaryDirectory() as d:
        fout = os.path.join(d, "out.bin")
        subprocess.run([HARNESS, "tsp", path, fout, "x"], check=True,
                       stdout=subprocess.DEVNULL)
        with open(fout, "rb") as f:
            b = f.read()
    (n,) = struct.unpack_from("<I", b, 0)
    return np.frombuffer(b, dtype=np.float32, count=2 * n, offset=4).reshape(n, 2).copy()


def step(xy, route):
    """One optimizeStep of the nint solver: (minchange, i, j)."""
    return struct.unpack_from("<iii", _run("step", xy, route), 0)
