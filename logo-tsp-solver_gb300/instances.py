"""Seeded instance and start-tour generators.

The reference draws everything from ``rand()`` seeded by the wall clock
(src/utils/common.c:253-259) and shuffles start tours with ``random_shuffle``
(src/utils/construction.c:135-137), so no run of it is reproducible.  These
generators replace that with SplitMix64 (Steele, Lea, Flood, OOPSLA 2014), the
same generator the device ILS and the oracle use, so every instance, start tour
and kick sequence is a function of a recorded seed.

All arithmetic is numpy elementwise IEEE (no reductions whose order could vary
across machines), so the x86 container and the Arm GPU host produce the same
bits.
"""
import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_STREAM = 0xD1B54A32D192ED03  # separates the streams drawn from one seed


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def splitmix64(seed, count, stream=0):
    """The first `count` SplitMix64 outputs from state seed + stream*C."""
    with np.errstate(over="ignore"):
        s = np.uint64((int(seed) + int(stream) * _STREAM) & ((1 << 64) - 1))
        k = np.arange(1, count + 1, dtype=np.uint64)
        return _mix(s + k * GAMMA)


def splitmix64_scalar(state):
    """One step on a Python int state; returns (output, new_state)."""
    state = (state + 0x9E3779B97F4A7C15) & ((1 << 64) - 1)
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & ((1 << 64) - 1)
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & ((1 << 64) - 1)
    return z ^ (z >> 31), state


def _unit24(u):
    """float32 in [0, 1) from the top 24 bits (exact)."""
    return (u >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)


def _unit53(u):
    """float64 in [0, 1) from the top 53 bits (exact)."""
    return (u >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def uniform_int(n, seed, side=10000):
    """n cities with integer coordinates uniform in [0, side)^2, as float32
    (the plain single-instance workload: n=1000, side=10000)."""
    u = splitmix64(seed, 2 * n, stream=1)
    v = ((u >> np.uint64(32)) % np.uint64(side)).astype(np.float32)
    return np.ascontiguousarray(v.reshape(n, 2))


def uniform_f32(n, seed, side):
    """n cities with float32 coordinates uniform in [0, side)^2."""
    u = splitmix64(seed, 2 * n, stream=2)
    v = _unit24(u) * np.float32(side)
    top = np.nextafter(np.float32(side), np.float32(0))
    v = np.minimum(v, top)
    return np.ascontiguousarray(v.reshape(n, 2).astype(np.float32))


def clustered(n, seed, side=1.0e6, clusters=200, sigma_frac=0.01):
    """Gaussian mixture: `clusters` centres uniform in [0, side)^2; each city
    picks a centre uniformly and adds N(0, (sigma_frac*side)^2) per axis,
    clamped to [0, side).  The normal deviate is the Irwin-Hall sum of 12
    uniforms minus 6 (mean 0, variance 1), which needs no libm call and so is
    bit-identical on every host."""
    cu = splitmix64(seed, 2 * clusters, stream=3)
    centres = (_unit53(cu) * side).reshape(clusters, 2)
    pick = splitmix64(seed, n, stream=4)
    idx = ((pick >> np.uint64(32)) % np.uint64(clusters)).astype(np.int64)
    g = splitmix64(seed, 24 * n, stream=5).reshape(n, 2, 12)
    z = np.zeros((n, 2), dtype=np.float64)
    for t in range(12):
        z = z + _unit53(g[:, :, t])
    z = z - 6.0
    pts = centres[idx] + (sigma_frac * side) * z
    pts = np.clip(pts, 0.0, side)
    p32 = pts.astype(np.float32)
    top = np.nextafter(np.float32(side), np.float32(0))
    p32 = np.minimum(p32, top)
    return np.ascontiguousarray(p32)


def random_tour(n, seed):
    """Fisher-Yates permutation of 0..n-1 driven by SplitMix64 (the seeded
    stand-in for random_shuffle, src/utils/construction.c:135-137)."""
    u = splitmix64(seed, max(n - 1, 0), stream=6)
    hi = (u >> np.uint64(32)).astype(np.uint64)
    p = np.arange(n, dtype=np.uint32)
    ks = np.arange(n - 1, 0, -1, dtype=np.uint64)
    js = ((hi[: n - 1] * (ks + np.uint64(1))) >> np.uint64(32)).astype(np.int64)
    pl = p.tolist()
    for t, k in enumerate(range(n - 1, 0, -1)):
        j = int(js[t])
        pl[k], pl[j] = pl[j], pl[k]
    return np.array(pl, dtype=np.uint32)


def batch_sizes(count, seed, n_lo=50, n_hi=2000):
    """n = round(exp(U(ln n_lo, ln n_hi))) for each of `count` instances."""
    u = _unit53(splitmix64(seed, count, stream=7))
    lo, hi = np.log(float(n_lo)), np.log(float(n_hi))
    # exp/log are libm calls: round to the nearest integer, which absorbs any
    # last-bit difference between hosts except at exact .5 ties
    ns = np.rint(np.exp(lo + (hi - lo) * u)).astype(np.int64)
    return np.clip(ns, n_lo, n_hi).astype(np.uint32)


def instance_seed(seed, k):
    """Per-instance seed k of a batch drawn from one master seed."""
    return int(splitmix64(seed, k + 1, stream=8)[k])


def batched_workload(count, seed, n_lo=50, n_hi=2000, side=1.0e4):
    """The batched workload: `count` instances with n log-uniform in
    [n_lo, n_hi], uniform float32 coordinates in [0, side)^2 and random start
    tours.  Returns (coords_list, routes, ils_seeds)."""
    ns = batch_sizes(count, seed, n_lo, n_hi)
    coords, routes, seeds = [], [], []
    for k in range(count):
        s = instance_seed(seed, k)
        coords.append(uniform_f32(int(ns[k]), s, side))
        routes.append(random_tour(int(ns[k]), s))
        seeds.append(s)
    return coords, routes, seeds
