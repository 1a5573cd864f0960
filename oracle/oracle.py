"""ctypes binding of the CPU oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` load
this module; the product library never does.  Every function mirrors one in
``oracle.h``, which cites the reference file:line each restates.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liblogo_oracle.so")
_lib = None

KICK_SEGMENT = 0
KICK_DOUBLE_BRIDGE = 1
NO_MOVE = (1 << 64) - 1

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)


class IlsStats(ctypes.Structure):
    _fields_ = [("moves", ctypes.c_uint64), ("descents", ctypes.c_uint64),
                ("accepted", ctypes.c_uint64), ("start_length", ctypes.c_uint64),
                ("best_length", ctypes.c_uint64)]


def build():
    """Compile liblogo_oracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.lo_dist.restype = ctypes.c_int32
        L.lo_dist.argtypes = [ctypes.c_float] * 4
        L.lo_splitmix64.restype = ctypes.c_uint64
        L.lo_splitmix64.argtypes = [_u64p]
        L.lo_uniform.restype = ctypes.c_uint32
        L.lo_uniform.argtypes = [_u64p, ctypes.c_uint32]
        L.lo_pack_key.restype = ctypes.c_uint64
        L.lo_pack_key.argtypes = [ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32]
        L.lo_best_move.restype = ctypes.c_int
        L.lo_best_move.argtypes = [_f32p, _u32p, ctypes.c_uint32, _i32p, _u32p, _u32p]
        L.lo_best_move_rows.restype = ctypes.c_uint64
        L.lo_best_move_rows.argtypes = [_f32p, _u32p, ctypes.c_uint32,
                                        ctypes.c_uint32, ctypes.c_uint32]
        L.lo_best_move_mt.restype = ctypes.c_uint64
        L.lo_best_move_mt.argtypes = [_f32p, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_uint32, ctypes.c_int]
        L.lo_apply_move.restype = None
        L.lo_apply_move.argtypes = [_u32p, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, _u32p]
        L.lo_tour_length.restype = ctypes.c_uint64
        L.lo_tour_length.argtypes = [_f32p, _u32p, ctypes.c_uint32]
        L.lo_descend.restype = ctypes.c_int64
        L.lo_descend.argtypes = [_f32p, _u32p, ctypes.c_uint32, ctypes.c_uint64,
                                 _i32p, ctypes.c_uint64]
        L.lo_descend_mt.restype = ctypes.c_int64
        L.lo_descend_mt.argtypes = [_f32p, _u32p, ctypes.c_uint32, ctypes.c_uint64,
                                    _i32p, ctypes.c_uint64, ctypes.c_int]
        L.lo_ils_mt.restype = ctypes.c_int
        L.lo_ils_mt.argtypes = [_f32p, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64,
                                ctypes.POINTER(IlsStats), ctypes.c_int]
        L.lo_kick_segment.restype = None
        L.lo_kick_segment.argtypes = [_u32p, ctypes.c_uint32, _u64p, _u32p]
        L.lo_kick_double_bridge.restype = None
        L.lo_kick_double_bridge.argtypes = [_u32p, ctypes.c_uint32, _u64p, _u32p]
        L.lo_ils.restype = ctypes.c_int
        L.lo_ils.argtypes = [_f32p, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                             ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64,
                             ctypes.POINTER(IlsStats)]
        L.lo_nn_tour.restype = ctypes.c_uint64
        L.lo_nn_tour.argtypes = [_f32p, ctypes.c_uint32, _u32p]
        L.lo_check_tour.restype = ctypes.c_int
        L.lo_check_tour.argtypes = [_u32p, ctypes.c_uint32]
        L.lo_knn.restype = ctypes.c_int
        L.lo_knn.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32, _u32p]
        L.lo_descend_nbr.restype = ctypes.c_int64
        L.lo_descend_nbr.argtypes = [_f32p, _u32p, ctypes.c_uint32, _u32p, ctypes.c_uint32,
                                     ctypes.c_uint64, ctypes.c_int, _u64p, ctypes.c_int]
        L.lo_nbr_step.restype = ctypes.c_int
        L.lo_nbr_step.argtypes = [_f32p, _u32p, ctypes.c_uint32, _u32p, ctypes.c_uint32,
                                  ctypes.c_int, _i32p, _i32p, _u32p, _u32p]
        L.lo_ils_nbr.restype = ctypes.c_int
        L.lo_ils_nbr.argtypes = [_f32p, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64,
                                 ctypes.POINTER(IlsStats), ctypes.c_int, _u32p,
                                 ctypes.c_uint32, ctypes.c_int]
        L.lo_ils_batch.restype = ctypes.c_int
        L.lo_ils_batch.argtypes = [_f32p, _u32p, _u64p, _u32p, _u64p, ctypes.c_uint32,
                                   ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                   _u64p, _u64p]
        _lib = L
    return _lib


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_f32p)


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(_u32p)


def dist(ax, ay, bx, by):
    return lib().lo_dist(ax, ay, bx, by)


def unpack_key(key):
    if key == NO_MOVE:
        return (0, 0, 0)
    return ((key >> 42) - (1 << 22), (key >> 21) & 0x1FFFFF, key & 0x1FFFFF)


def pack_key(delta, i, j):
    return lib().lo_pack_key(delta, i, j)


def best_move(xy, route):
    """(delta, i, j) of the best move, (0, 0, 0) if none (reference best2_out)."""
    xy, pxy = _f32(xy)
    route, pr = _u32(route)
    d = ctypes.c_int32()
    i = ctypes.c_uint32()
    j = ctypes.c_uint32()
    rc = lib().lo_best_move(pxy, pr, len(route), ctypes.byref(d), ctypes.byref(i),
                            ctypes.byref(j))
    if rc < 0:
        raise MemoryError("oracle sweep allocation failed")
    return (d.value, i.value, j.value)


def best_move_key(xy, route, row_lo=1, row_hi=0, threads=1):
    xy, pxy = _f32(xy)
    route, pr = _u32(route)
    if threads > 1:
        return lib().lo_best_move_mt(pxy, pr, len(route), row_lo, row_hi, threads)
    return lib().lo_best_move_rows(pxy, pr, len(route), row_lo, row_hi)


def apply_move(route, i, j):
    r = np.array(route, dtype=np.uint32, copy=True)
    tmp = np.empty_like(r)
    lib().lo_apply_move(r.ctypes.data_as(_u32p), len(r), i, j, tmp.ctypes.data_as(_u32p))
    return r


def tour_length(xy, route):
    xy, pxy = _f32(xy)
    route, pr = _u32(route)
    return lib().lo_tour_length(pxy, pr, len(route))


def knn(xy, k):
    """(n, k) uint32: the k nearest other cities of every city (squared
    double distance, lower id on ties; brute force)."""
    xy, pxy = _f32(xy)
    n = len(xy)
    out = np.zeros((n, k), dtype=np.uint32)
    if lib().lo_knn(pxy, n, k, out.ctypes.data_as(_u32p)):
        raise MemoryError("oracle knn allocation failed")
    return out


def descend_nbr(xy, route, k=8, max_moves=None, threads=1, stop_at_limit=False, oropt=False):
    """Neighbour-list search (neighbour moves, then full sweeps): returns
    (final_route, moves, moves of the neighbour phase).  stop_at_limit: a
    descent that still has moves after max_moves returns its state there
    (moves = max_moves) instead of raising."""
    nb = np.ascontiguousarray(knn(xy, k))
    xy, pxy = _f32(xy)
    r = np.array(route, dtype=np.uint32, copy=True)
    n = len(r)
    if max_moves is None:
        max_moves = 64 * n * n + 1024
    nm = ctypes.c_uint64(0)
    m = lib().lo_descend_nbr(pxy, r.ctypes.data_as(_u32p), n, nb.ctypes.data_as(_u32p), k,
                             max_moves, max(1, int(threads)), ctypes.byref(nm), int(oropt))
    if m < 0:
        if not stop_at_limit:
            raise RuntimeError("oracle descent exceeded max_moves")
        m = max_moves
    return r, m, nm.value


def nbr_step(xy, route, k=8, oropt=False, nb=None):
    """The move one neighbour-search step would apply: (delta, slot, i, j)
    with slot -1 for 2-opt, else the Or-opt variant; None if none improves."""
    if nb is None:
        nb = knn(xy, k)
    nb = np.ascontiguousarray(nb, dtype=np.uint32)
    xy, pxy = _f32(xy)
    route, pr = _u32(route)
    d, sl = ctypes.c_int32(), ctypes.c_int32()
    i, j = ctypes.c_uint32(), ctypes.c_uint32()
    rc = lib().lo_nbr_step(pxy, pr, len(route), nb.ctypes.data_as(_u32p), k, int(oropt),
                           ctypes.byref(d), ctypes.byref(sl), ctypes.byref(i), ctypes.byref(j))
    if rc < 0:
        raise MemoryError("oracle allocation failed")
    return None if rc == 1 else (d.value, sl.value, i.value, j.value)


def ils_nbr(xy, route, kicks, seed, kind=KICK_SEGMENT, k=8, max_moves=None, threads=1,
            oropt=False):
    """ils() with the neighbour-list search in every descent."""
    nb = np.ascontiguousarray(knn(xy, k))
    xy, pxy = _f32(xy)
    r = np.array(route, dtype=np.uint32, copy=True)
    n = len(r)
    if max_moves is None:
        max_moves = 64 * n * n + 1024
    st = IlsStats()
    rc = lib().lo_ils_nbr(pxy, r.ctypes.data_as(_u32p), n, kicks, seed, kind, max_moves,
                          ctypes.byref(st), max(1, int(threads)), nb.ctypes.data_as(_u32p), k,
                          int(oropt))
    if rc:
        raise RuntimeError("oracle ILS descent exceeded max_moves")
    return r, {f: getattr(st, f) for f, _ in IlsStats._fields_}


def descend(xy, route, max_moves=None, log_cap=0, threads=1):
    """Returns (final_route, moves, log) where log is an (m, 3) int32 array.
    threads > 1 splits every sweep over that many host threads (same moves)."""
    xy, pxy = _f32(xy)
    r = np.array(route, dtype=np.uint32, copy=True)
    n = len(r)
    if max_moves is None:
        max_moves = 64 * n * n + 1024
    log = np.zeros((max(log_cap, 1), 3), dtype=np.int32)
    m = lib().lo_descend_mt(pxy, r.ctypes.data_as(_u32p), n, max_moves,
                            log.ctypes.data_as(_i32p), log_cap, max(1, int(threads)))
    if m < 0:
        raise RuntimeError("oracle descent exceeded max_moves")
    return r, m, log[: min(m, log_cap)]


def kick(route, rng_state, kind=KICK_SEGMENT):
    """Applies one kick; returns (new_route, new_rng_state)."""
    r = np.array(route, dtype=np.uint32, copy=True)
    tmp = np.empty_like(r)
    st = ctypes.c_uint64(rng_state)
    fn = lib().lo_kick_double_bridge if kind == KICK_DOUBLE_BRIDGE else lib().lo_kick_segment
    fn(r.ctypes.data_as(_u32p), len(r), ctypes.byref(st), tmp.ctypes.data_as(_u32p))
    return r, st.value


def ils(xy, route, kicks, seed, kind=KICK_SEGMENT, max_moves=None, threads=1):
    xy, pxy = _f32(xy)
    r = np.array(route, dtype=np.uint32, copy=True)
    n = len(r)
    if max_moves is None:
        max_moves = 64 * n * n + 1024
    st = IlsStats()
    rc = lib().lo_ils_mt(pxy, r.ctypes.data_as(_u32p), n, kicks, seed, kind, max_moves,
                         ctypes.byref(st), max(1, int(threads)))
    if rc:
        raise RuntimeError("oracle ILS descent exceeded max_moves")
    return r, {k: getattr(st, k) for k, _ in IlsStats._fields_}


def ils_batch(xy_list, routes, seeds, kicks, kind=KICK_SEGMENT, threads=1):
    """ILS over many instances on `threads` host threads. Returns
    (routes, best_lengths, moves)."""
    ns = np.array([len(r) for r in routes], dtype=np.uint32)
    offs = np.zeros(len(routes), dtype=np.uint64)
    offs[1:] = np.cumsum(ns[:-1].astype(np.uint64))
    xy = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float32).reshape(-1)
                                              for a in xy_list]))
    rr = np.ascontiguousarray(np.concatenate([np.asarray(r, np.uint32) for r in routes]))
    sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
    lens = np.zeros(len(routes), dtype=np.uint64)
    mv = np.zeros(len(routes), dtype=np.uint64)
    rc = lib().lo_ils_batch(xy.ctypes.data_as(_f32p), rr.ctypes.data_as(_u32p),
                            offs.ctypes.data_as(_u64p), ns.ctypes.data_as(_u32p),
                            sd.ctypes.data_as(_u64p), len(routes), kicks, kind, threads,
                            lens.ctypes.data_as(_u64p), mv.ctypes.data_as(_u64p))
    if rc:
        raise RuntimeError("oracle batch ILS failed")
    out = [rr[int(o):int(o) + int(n)].copy() for o, n in zip(offs, ns)]
    return out, lens, mv


def nn_tour(xy):
    """Returns (route, ties)."""
    xy, pxy = _f32(xy)
    n = xy.size // 2
    r = np.zeros(n, dtype=np.uint32)
    ties = lib().lo_nn_tour(pxy, n, r.ctypes.data_as(_u32p))
    return r, ties


def check_tour(route, n=None):
    route, pr = _u32(route)
    return bool(lib().lo_check_tour(pr, len(route) if n is None else n))


def splitmix_sequence(seed, count):
    st = ctypes.c_uint64(seed)
    return [lib().lo_splitmix64(ctypes.byref(st)) for _ in range(count)]
