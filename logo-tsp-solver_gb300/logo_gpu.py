"""Python binding of the C ABI in include/logo_gpu.h (ctypes, no torch).

The library is liblogo_gpu.so built in this directory by build_lib.py.  There
is no CPU fallback: if the library cannot be loaded, or no CUDA device is
present, calls raise.

The class names mirror the reference's solver interface:
  Solver.optimize_step  ≙ LocalSolver::optimizeStep (src/solvers/localSolver.h:124-125)
  Solver.optimize       ≙ TwoOptLocalSolver::optimize (src/solvers/twoOptLocalSolver.cpp:22-64)
  Solver.ils            ≙ ILSGlobalSolverSequential::optimize
                          (src/solvers/ILSGlobalSolverSequential.cpp:60-100)
  Solver.route_length   ≙ routeLength (src/headers.h:170-189)
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblogo_gpu.so")

KICK_SEGMENT = 0
KICK_DOUBLE_BRIDGE = 1
SWEEP_MUFU = 0
SWEEP_FUSED = 4
SWEEP_LOCAL = 5
SWEEP_BOXED = 6
DESCENT_AUTO = 0
DESCENT_GRAPH = 1
DESCENT_COOPERATIVE = 2
ROUTE_IO_AUTO = 0
ROUTE_IO_COPY = 1
ROUTE_IO_DIRECT = 2
SEARCH_EXHAUSTIVE = 0
SEARCH_NEIGHBOUR = 1
SEARCH_NEIGHBOUR_OROPT = 2
START_GIVEN = 0
START_NN = 1
START_MF = 2
MAX_CITIES = 2097152

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA", 4: "TIMEOUT", 5: "DEVICE_FAULT",
          6: "MOVE_LIMIT", 7: "NO_DEVICE", 8: "BUSY", 9: "NOT_FOUND"}

# every exported symbol of include/logo_gpu.h (checked by the CPU test suite)
EXPORTS = [
    "logo_ctx_create", "logo_ctx_destroy", "logo_last_error", "logo_best_move",
    "logo_descend", "logo_ils", "logo_tour_length", "logo_set_route", "logo_get_route",
    "logo_descend_resident", "logo_sweep_resident", "logo_length_resident", "logo_sync",
    "logo_ctx_get_info", "logo_ctx_set_shape", "logo_ctx_stream", "logo_version",
    "logo_descend_trace", "logo_diag_sqrt_error", "logo_diag_wait_limits", "logo_begin_descent",
    "logo_enqueue_sweep", "logo_enqueue_apply", "logo_get_progress",
    "logo_read_tsplib", "logo_nn_tour", "logo_mf_tour", "logo_random_tour", "logo_check_tour",
    "logo_tsplib_info", "logo_read_tour", "logo_write_tour",
    "logo_batch_create", "logo_batch_destroy", "logo_batch_last_error", "logo_batch_run",
    "logo_batch_solve", "logo_batch_autotune", "logo_batch_shape_for", "logo_batch_multistart",
    "logo_best_move_noalloc", "logo_ctx_set_kernel", "logo_ctx_set_descent_mode",
    "logo_server_create", "logo_server_submit", "logo_server_poll", "logo_server_wait",
    "logo_server_get_stats", "logo_server_destroy", "logo_server_last_error",
    "logo_diag_flag_timeout", "logo_ctx_set_route_io", "logo_ctx_set_search",
    "logo_neighbours", "logo_start_tour",
]


class LogoError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Move(ctypes.Structure):
    """best2_out (src/defs.h:181-187)."""
    _fields_ = [("i", ctypes.c_uint32), ("j", ctypes.c_uint32), ("minchange", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("moves", ctypes.c_uint64), ("sweeps", ctypes.c_uint64),
                ("pair_evals", ctypes.c_uint64), ("descents", ctypes.c_uint64),
                ("kicks", ctypes.c_uint64), ("accepted", ctypes.c_uint64),
                ("start_length", ctypes.c_uint64), ("final_length", ctypes.c_uint64),
                ("device_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CtxInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("device", ctypes.c_int),
                ("rows_per_thread", ctypes.c_int), ("warps_per_cta", ctypes.c_int),
                ("tile_cols", ctypes.c_uint32), ("tiles", ctypes.c_uint32),
                ("filter_margin", ctypes.c_float), ("graph_steps", ctypes.c_uint32),
                ("variant", ctypes.c_int), ("descent_mode", ctypes.c_int),
                ("cooperative_ctas", ctypes.c_int), ("host_waits", ctypes.c_uint64),
                ("route_io", ctypes.c_int), ("search", ctypes.c_int),
                ("search_neighbours", ctypes.c_uint32), ("pad0", ctypes.c_uint32)]


class Instance(ctypes.Structure):
    _fields_ = [("coords", ctypes.c_void_p), ("route", ctypes.c_void_p),
                ("n", ctypes.c_uint32), ("seed", ctypes.c_uint64)]


class BatchShape(ctypes.Structure):
    _fields_ = [("rows_per_thread", ctypes.c_int), ("threads_per_cta", ctypes.c_int),
                ("tile_cols", ctypes.c_int)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("kicks", ctypes.c_uint32),
                ("kick_kind", ctypes.c_int), ("shape", BatchShape), ("ctas", ctypes.c_uint32),
                ("start", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("start_length", ctypes.c_uint64), ("best_length", ctypes.c_uint64),
                ("moves", ctypes.c_uint64), ("sweeps", ctypes.c_uint64),
                ("kicks", ctypes.c_uint32), ("accepted", ctypes.c_uint32),
                ("status", ctypes.c_int32), ("pad", ctypes.c_uint32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("mem_budget", ctypes.c_uint64),
                ("max_slots", ctypes.c_uint32), ("max_large", ctypes.c_uint32),
                ("kicks", ctypes.c_uint32), ("kick_kind", ctypes.c_int),
                ("quantum_pairs", ctypes.c_uint64), ("max_pending", ctypes.c_uint32)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("start_length", ctypes.c_uint64), ("best_length", ctypes.c_uint64),
                ("moves", ctypes.c_uint64), ("sweeps", ctypes.c_uint64),
                ("n", ctypes.c_uint32), ("kicks", ctypes.c_uint32),
                ("accepted", ctypes.c_uint32), ("status", ctypes.c_int32),
                ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("admitted", ctypes.c_uint64),
                ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("pending", ctypes.c_uint64), ("running_small", ctypes.c_uint64),
                ("running_large", ctypes.c_uint64), ("rounds", ctypes.c_uint64),
                ("round_device_ms", ctypes.c_double), ("mem_in_use", ctypes.c_uint64),
                ("mem_budget", ctypes.c_uint64)]


_lib = None
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p


def build(force=False):
    import importlib.util
    spec = importlib.util.spec_from_file_location("_logo_build_lib",
                                                  os.path.join(HERE, "build_lib.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build(force=force)


def load(path=LIB_PATH):
    """Loads liblogo_gpu.so (raises OSError if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    L = ctypes.CDLL(path)
    c = ctypes
    L.logo_version.restype = c.c_char_p
    L.logo_last_error.restype = c.c_char_p
    L.logo_last_error.argtypes = [_vp]
    L.logo_ctx_create.argtypes = [c.c_int, _vp, c.c_uint32, c.POINTER(_vp)]
    L.logo_ctx_destroy.argtypes = [_vp]
    L.logo_best_move.argtypes = [_vp, _u32p, c.POINTER(Move)]
    L.logo_descend.argtypes = [_vp, _u32p, c.c_uint64, c.POINTER(Stats)]
    L.logo_ils.argtypes = [_vp, _u32p, c.c_uint32, c.c_uint64, c.c_int, c.POINTER(Stats)]
    L.logo_tour_length.argtypes = [_vp, _u32p, _u64p]
    L.logo_set_route.argtypes = [_vp, _u32p]
    L.logo_get_route.argtypes = [_vp, _u32p]
    L.logo_descend_resident.argtypes = [_vp, c.c_uint64, c.POINTER(Stats)]
    L.logo_sweep_resident.argtypes = [_vp, c.POINTER(Move)]
    L.logo_length_resident.argtypes = [_vp, _u64p]
    L.logo_sync.argtypes = [_vp]
    L.logo_ctx_get_info.argtypes = [_vp, c.POINTER(CtxInfo)]
    L.logo_ctx_set_shape.argtypes = [_vp, c.c_int, c.c_int, c.c_uint32]
    L.logo_ctx_set_kernel.argtypes = [_vp, c.c_int, c.c_int, c.c_int, c.c_uint32]
    L.logo_ctx_set_descent_mode.argtypes = [_vp, c.c_int]
    L.logo_ctx_set_route_io.argtypes = [_vp, c.c_int]
    L.logo_ctx_set_search.argtypes = [_vp, c.c_int, c.c_uint32]
    L.logo_start_tour.argtypes = [_vp, c.c_int, _u32p]
    L.logo_ctx_stream.restype = _vp
    L.logo_ctx_stream.argtypes = [_vp]
    L.logo_descend_trace.argtypes = [_vp, _u32p, c.c_uint64, ctypes.POINTER(ctypes.c_int32),
                                     c.c_uint64, c.POINTER(Stats)]
    L.logo_diag_sqrt_error.argtypes = [c.c_int, ctypes.POINTER(ctypes.c_double)]
    L.logo_diag_flag_timeout.argtypes = [_vp]
    L.logo_diag_wait_limits.argtypes = [c.c_int, ctypes.POINTER(ctypes.c_uint32),
                                        ctypes.POINTER(ctypes.c_uint32),
                                        ctypes.POINTER(ctypes.c_double)]
    L.logo_begin_descent.argtypes = [_vp, c.c_uint64]
    L.logo_enqueue_sweep.argtypes = [_vp]
    L.logo_enqueue_apply.argtypes = [_vp]
    L.logo_get_progress.argtypes = [_vp, _u64p, ctypes.POINTER(ctypes.c_int)]
    L.logo_read_tsplib.argtypes = [c.c_char_p, _vp, c.c_uint32, _u32p]
    L.logo_nn_tour.argtypes = [_vp, c.c_uint32, c.c_uint32, _u32p]
    L.logo_mf_tour.argtypes = [_vp, c.c_uint32, _u32p]
    L.logo_neighbours.argtypes = [_vp, c.c_uint32, c.c_uint32, _u32p]
    L.logo_tsplib_info.argtypes = [c.c_char_p, _u32p, c.POINTER(c.c_int)]
    L.logo_read_tour.argtypes = [c.c_char_p, _u32p, c.c_uint32, _u32p]
    L.logo_write_tour.argtypes = [c.c_char_p, _u32p, c.c_uint32, c.c_char_p, c.c_int]
    L.logo_random_tour.argtypes = [c.c_uint32, c.c_uint64, _u32p]
    L.logo_check_tour.argtypes = [_u32p, c.c_uint32]
    L.logo_batch_create.argtypes = [c.c_int, c.c_uint32, c.c_uint64, c.POINTER(_vp)]
    L.logo_batch_destroy.argtypes = [_vp]
    L.logo_batch_last_error.restype = c.c_char_p
    L.logo_batch_last_error.argtypes = [_vp]
    L.logo_batch_run.argtypes = [_vp, _vp, c.c_uint32, c.POINTER(BatchOpts), _vp,
                                 c.POINTER(c.c_double)]
    L.logo_batch_solve.argtypes = [_vp, c.c_uint32, c.POINTER(BatchOpts), _vp,
                                   c.POINTER(c.c_double)]
    L.logo_batch_autotune.argtypes = [_vp, _vp, c.c_uint32, c.c_uint32, c.c_int, c.c_char_p,
                                      c.c_int]
    L.logo_batch_shape_for.argtypes = [_vp, c.c_uint32, c.POINTER(BatchShape)]
    L.logo_batch_multistart.argtypes = [_vp, _vp, c.c_uint32, _u32p, c.c_uint32, c.c_uint64,
                                        c.c_int, c.POINTER(BatchOpts), _vp,
                                        c.POINTER(c.c_uint32), c.POINTER(c.c_double)]
    L.logo_best_move_noalloc.argtypes = [_vp, _vp, c.c_uint32, _vp, _vp, _vp]
    L.logo_server_create.argtypes = [c.POINTER(ServerOpts), c.POINTER(_vp)]
    L.logo_server_submit.argtypes = [_vp, _vp, c.c_uint32, _u32p, c.c_uint64, _u64p]
    L.logo_server_poll.argtypes = [_vp, c.c_uint64, _u32p, c.POINTER(RequestInfo)]
    L.logo_server_wait.argtypes = [_vp, c.c_uint64, c.c_uint32, _u32p, c.POINTER(RequestInfo)]
    L.logo_server_get_stats.argtypes = [_vp, c.POINTER(ServerStats)]
    L.logo_server_destroy.argtypes = [_vp]
    L.logo_server_last_error.restype = c.c_char_p
    L.logo_server_last_error.argtypes = [_vp]
    _lib = L
    return L


def _check(status, ctx=None):
    if status != 0:
        msg = load().logo_last_error(ctx).decode(errors="replace")
        raise LogoError(status, msg)


def _route_arg(route, n):
    r = np.ascontiguousarray(route, dtype=np.uint32)
    if r.shape != (n,):
        raise ValueError(f"route must have shape ({n},)")
    return r


class Solver:
    """One instance on one GPU (a logo_ctx)."""

    def __init__(self, coords, device=0):
        L = load()
        xy = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 2)
        self.n = xy.shape[0]
        self._xy = xy
        h = _vp()
        _check(L.logo_ctx_create(device, xy.ctypes.data, self.n, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().logo_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- reference-shaped API ------------------------------------------------
    def optimize_step(self, route):
        """(minchange, i, j) of the best move (best2_out)."""
        r = _route_arg(route, self.n)
        m = Move()
        _check(load().logo_best_move(self._h, r.ctypes.data_as(_u32p), ctypes.byref(m)),
               self._h)
        return (m.minchange, m.i, m.j)

    def optimize(self, route, max_moves=0, stats=True, out=None):
        """2-opt descent; returns (route, stats).  With stats=False no length
        is computed (stats is None); `out` may supply the result array."""
        r = out if out is not None else np.empty(self.n, dtype=np.uint32)
        r[:] = route
        _route_arg(r, self.n)
        st = Stats() if stats else None
        _check(load().logo_descend(self._h, r.ctypes.data_as(_u32p), max_moves,
                                   ctypes.byref(st) if stats else None), self._h)
        return r, (st.as_dict() if stats else None)

    def optimize_inplace(self, route, max_moves=0, stats=False):
        """2-opt descent on `route` itself (a C-contiguous uint32 array of
        length n, rewritten with the result), as the reference's
        LocalSolver::optimize(route) works on the caller's buffer: the
        C-ABI call with no copy on the Python side.  Returns the stats dict
        or None."""
        if (not isinstance(route, np.ndarray) or route.dtype != np.uint32 or
                route.shape != (self.n,) or not route.flags.c_contiguous or
                not route.flags.writeable):
            raise ValueError(f"route must be a writeable C-contiguous uint32 array of shape ({self.n},)")
        st = Stats() if stats else None
        _check(load().logo_descend(self._h, route.ctypes.data_as(_u32p), max_moves,
                                   ctypes.byref(st) if stats else None), self._h)
        return st.as_dict() if stats else None

    def optimize_trace(self, route, max_moves=0, trace_cap=1 << 20):
        """Descent that also returns the (minchange, i, j) of every move."""
        r = np.array(route, dtype=np.uint32, copy=True)
        _route_arg(r, self.n)
        tr = np.zeros((trace_cap, 3), dtype=np.int32)
        st = Stats()
        _check(load().logo_descend_trace(self._h, r.ctypes.data_as(_u32p), max_moves,
                                         tr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                         trace_cap, ctypes.byref(st)), self._h)
        return r, tr[: min(st.moves, trace_cap)].copy(), st.as_dict()

    def ils(self, route, kicks, seed, kind=KICK_SEGMENT):
        r = np.array(route, dtype=np.uint32, copy=True)
        _route_arg(r, self.n)
        st = Stats()
        _check(load().logo_ils(self._h, r.ctypes.data_as(_u32p), kicks, seed, kind,
                               ctypes.byref(st)), self._h)
        return r, st.as_dict()

    def route_length(self, route):
        r = _route_arg(route, self.n)
        v = ctypes.c_uint64()
        _check(load().logo_tour_length(self._h, r.ctypes.data_as(_u32p), ctypes.byref(v)),
               self._h)
        return v.value

    # -- resident tour ----------------------------------------------------------
    def set_route(self, route):
        r = _route_arg(route, self.n)
        _check(load().logo_set_route(self._h, r.ctypes.data_as(_u32p)), self._h)

    def get_route(self):
        r = np.zeros(self.n, dtype=np.uint32)
        _check(load().logo_get_route(self._h, r.ctypes.data_as(_u32p)), self._h)
        return r

    def descend_resident(self, max_moves=0):
        st = Stats()
        _check(load().logo_descend_resident(self._h, max_moves, ctypes.byref(st)), self._h)
        return st.as_dict()

    def sweep_resident(self):
        m = Move()
        _check(load().logo_sweep_resident(self._h, ctypes.byref(m)), self._h)
        return (m.minchange, m.i, m.j)

    def length_resident(self):
        v = ctypes.c_uint64()
        _check(load().logo_length_resident(self._h, ctypes.byref(v)), self._h)
        return v.value

    def sync(self):
        _check(load().logo_sync(self._h), self._h)

    # -- stream-ordered primitives ----------------------------------------------
    def begin_descent(self, max_moves=0):
        _check(load().logo_begin_descent(self._h, max_moves), self._h)

    def enqueue_sweep(self):
        _check(load().logo_enqueue_sweep(self._h), self._h)

    def enqueue_apply(self):
        _check(load().logo_enqueue_apply(self._h), self._h)

    def progress(self):
        m = ctypes.c_uint64()
        cv = ctypes.c_int()
        _check(load().logo_get_progress(self._h, ctypes.byref(m), ctypes.byref(cv)), self._h)
        return m.value, bool(cv.value)

    def info(self):
        i = CtxInfo()
        _check(load().logo_ctx_get_info(self._h, ctypes.byref(i)), self._h)
        return {k: getattr(i, k) for k, _ in CtxInfo._fields_}

    def set_kernel(self, variant, rows_per_thread, warps_per_cta, tile_cols):
        """Variant (SWEEP_MUFU .. SWEEP_BOXED) and tile shape."""
        _check(load().logo_ctx_set_kernel(self._h, variant, rows_per_thread, warps_per_cta,
                                          tile_cols), self._h)

    def set_descent_mode(self, mode):
        """DESCENT_AUTO, DESCENT_GRAPH or DESCENT_COOPERATIVE."""
        _check(load().logo_ctx_set_descent_mode(self._h, mode), self._h)

    def set_route_io(self, mode):
        """ROUTE_IO_AUTO, ROUTE_IO_COPY or ROUTE_IO_DIRECT (how route buffers
        reach the device; info()["route_io"] gives the mode in use)."""
        _check(load().logo_ctx_set_route_io(self._h, mode), self._h)

    def start_tour(self, kind=START_NN):
        """The instance's START_NN or START_MF tour built on the device
        (n <= 4096)."""
        r = np.zeros(self.n, dtype=np.uint32)
        _check(load().logo_start_tour(self._h, kind, r.ctypes.data_as(_u32p)), self._h)
        return r

    def set_search(self, mode, neighbours=0):
        """SEARCH_EXHAUSTIVE (the reference's best improvement) or
        SEARCH_NEIGHBOUR (neighbour-list moves first, then full sweeps to a
        2-opt local optimum); neighbours 1..16, 0 = 8."""
        _check(load().logo_ctx_set_search(self._h, mode, neighbours), self._h)

    def set_shape(self, rows_per_thread, warps_per_cta, tile_cols):
        _check(load().logo_ctx_set_shape(self._h, rows_per_thread, warps_per_cta, tile_cols),
               self._h)

    @property
    def stream(self):
        return load().logo_ctx_stream(self._h)

    def flag_timeout(self):
        """Test hook: marks the context's device status as a timed-out wait
        would (logo_diag_flag_timeout)."""
        _check(load().logo_diag_flag_timeout(self._h), self._h)


def read_tsplib(path):
    """TSPLIB coordinates as an (n, 2) float32 array (host only)."""
    L = load()
    n = ctypes.c_uint32()
    _check(L.logo_read_tsplib(os.fsencode(path), None, 0, ctypes.byref(n)))
    xy = np.zeros((n.value, 2), dtype=np.float32)
    _check(L.logo_read_tsplib(os.fsencode(path), xy.ctypes.data, n.value, ctypes.byref(n)))
    return xy


def nn_tour(coords, start=0):
    """Nearest-neighbour start tour (host only)."""
    xy = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 2)
    r = np.zeros(len(xy), dtype=np.uint32)
    _check(load().logo_nn_tour(xy.ctypes.data, len(xy), start, r.ctypes.data_as(_u32p)))
    return r


def neighbours(coords, k):
    """(n, k) uint32: the k nearest other cities of every city (the
    candidate lists of SEARCH_NEIGHBOUR; host only)."""
    xy = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 2)
    out = np.zeros((len(xy), k), dtype=np.uint32)
    _check(load().logo_neighbours(xy.ctypes.data, len(xy), k, out.ctypes.data_as(_u32p)))
    return out


def mf_tour(coords):
    """Multiple-fragment (greedy edge) start tour (host only)."""
    xy = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 2)
    r = np.zeros(len(xy), dtype=np.uint32)
    _check(load().logo_mf_tour(xy.ctypes.data, len(xy), r.ctypes.data_as(_u32p)))
    return r


EDGE_WEIGHT_TYPES = {0: "EUC_2D", 1: "CEIL_2D", 2: "ATT", 3: "GEO", 4: "OTHER"}


def tsplib_info(path):
    """(dimension, EDGE_WEIGHT_TYPE name) of a TSPLIB file."""
    n, t = ctypes.c_uint32(), ctypes.c_int()
    _check(load().logo_tsplib_info(os.fsencode(path), ctypes.byref(n), ctypes.byref(t)))
    return n.value, EDGE_WEIGHT_TYPES[t.value]


def read_tour(path):
    """A tour file (TSPLIB .tour or a bare id list, 1-based) as 0-based ids."""
    n = ctypes.c_uint32()
    _check(load().logo_read_tour(os.fsencode(path), None, 0, ctypes.byref(n)))
    r = np.zeros(n.value, dtype=np.uint32)
    _check(load().logo_read_tour(os.fsencode(path), r.ctypes.data_as(_u32p), n.value,
                                 ctypes.byref(n)))
    return r


def write_tour(path, route, name="tour", tsplib_header=True):
    r = np.ascontiguousarray(route, dtype=np.uint32)
    _check(load().logo_write_tour(os.fsencode(path), r.ctypes.data_as(_u32p), len(r),
                                  name.encode(), int(bool(tsplib_header))))


def random_tour(n, seed):
    r = np.zeros(n, dtype=np.uint32)
    _check(load().logo_random_tour(n, seed, r.ctypes.data_as(_u32p)))
    return r


def check_tour(route):
    r = np.ascontiguousarray(route, dtype=np.uint32)
    return bool(load().logo_check_tour(r.ctypes.data_as(_u32p), len(r)))


def sqrt_error(device=0):
    """Largest relative error of the device's approximate sqrt (see
    logo_diag_sqrt_error)."""
    v = ctypes.c_double()
    _check(load().logo_diag_sqrt_error(device, ctypes.byref(v)))
    return v.value


def wait_limits(device=0):
    """Runs two device waits that nothing satisfies (an mbarrier expecting
    bytes no copy delivers, the cooperative grid barrier missing a CTA) and
    returns (mbarrier_status, barrier_status, waited_ms); each status holds
    the timeout bit (1) when its wait gave up (see logo_diag_wait_limits)."""
    a, b, ms = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
    _check(load().logo_diag_wait_limits(device, ctypes.byref(a), ctypes.byref(b),
                                        ctypes.byref(ms)))
    return a.value, b.value, ms.value


def _batch_check(status, b):
    if status != 0:
        msg = load().logo_batch_last_error(b).decode(errors="replace")
        raise LogoError(status, msg)


class Batch:
    """Batched persistent solver (logo_batch).  solve() runs descent + ILS on
    every instance in one persistent launch per tile shape."""

    def __init__(self, max_count, max_cities, device=0):
        h = _vp()
        _batch_check(load().logo_batch_create(device, max_count, max_cities, ctypes.byref(h)),
                     None)
        self._h = h
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            load().logo_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def _pack(coords_list, routes, seeds):
        xs = [np.ascontiguousarray(c, dtype=np.float32).reshape(-1, 2) for c in coords_list]
        rs = [np.array(r, dtype=np.uint32, copy=True) for r in routes]
        arr = (Instance * len(xs))()
        for k, (x, r) in enumerate(zip(xs, rs)):
            arr[k].coords = x.ctypes.data
            arr[k].route = r.ctypes.data
            arr[k].n = len(r)
            arr[k].seed = int(seeds[k]) & ((1 << 64) - 1)
        return arr, xs, rs

    def solve(self, coords_list, routes, seeds, kicks=0, kind=KICK_SEGMENT, shape=None, ctas=0,
              start=START_GIVEN):
        """Returns (routes, results as a list of dicts, device_ms).  With
        start=START_NN or START_MF the routes are built on the device (routes may be None)."""
        if routes is None:
            routes = [np.zeros(len(np.asarray(c).reshape(-1, 2)), np.uint32) for c in coords_list]
        arr, xs, rs = self._pack(coords_list, routes, seeds)
        o = BatchOpts()
        o.device = self.device
        o.kicks = kicks
        o.kick_kind = kind
        o.start = start
        if shape:
            o.shape = BatchShape(*shape)
        o.ctas = ctas
        res = (Result * len(rs))()
        ms = ctypes.c_double()
        _batch_check(load().logo_batch_run(self._h, arr, len(rs), ctypes.byref(o), res,
                                           ctypes.byref(ms)), self._h)
        out = [{k: getattr(r, k) for k, _ in Result._fields_ if k != "pad"} for r in res]
        return rs, out, ms.value

    def multistart(self, coords, route, replicas, seed, share=True, kicks=0,
                   kind=KICK_SEGMENT):
        """Multi-start ILS of one instance: returns (best route, per-replica
        results, index of the replica returned, device_ms)."""
        xy = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 2)
        r = np.array(route, dtype=np.uint32, copy=True)
        o = BatchOpts()
        o.device = self.device
        o.kicks = kicks
        o.kick_kind = kind
        res = (Result * replicas)()
        best = ctypes.c_uint32()
        ms = ctypes.c_double()
        _batch_check(load().logo_batch_multistart(
            self._h, xy.ctypes.data, len(xy), r.ctypes.data_as(_u32p), replicas,
            int(seed) & ((1 << 64) - 1), int(bool(share)), ctypes.byref(o), res,
            ctypes.byref(best), ctypes.byref(ms)), self._h)
        out = [{k: getattr(x, k) for k, _ in Result._fields_ if k != "pad"} for x in res]
        return r, out, best.value, ms.value

    def autotune(self, coords_list, routes, seeds, kicks=0, kind=KICK_SEGMENT,
                 cache_path=None, reuse=False):
        arr, xs, rs = self._pack(coords_list, routes, seeds)
        _batch_check(load().logo_batch_autotune(
            self._h, arr, len(rs), kicks, kind,
            os.fsencode(cache_path) if cache_path else None, 1 if reuse else 0), self._h)

    def shape_for(self, n):
        s = BatchShape()
        _batch_check(load().logo_batch_shape_for(self._h, n, ctypes.byref(s)), self._h)
        return (s.rows_per_thread, s.threads_per_cta, s.tile_cols)


def best_move_noalloc(coords_ptr, route_ptr, n, out_ptr, status_ptr=None, stream=None):
    """logo_best_move_noalloc on caller-owned device pointers (ints); enqueues
    on `stream` (a cudaStream_t as int, None = legacy default stream)."""
    _check(load().logo_best_move_noalloc(coords_ptr, route_ptr, n, out_ptr, status_ptr,
                                         stream))


class Server:
    """Continuous-batching request server (logo_server)."""

    BUSY = 8

    def __init__(self, kicks=0, kind=KICK_SEGMENT, device=0, mem_budget=0, max_slots=0,
                 max_large=0, quantum_pairs=0, max_pending=0):
        o = ServerOpts(device, mem_budget, max_slots, max_large, kicks, kind, quantum_pairs,
                       max_pending)
        h = _vp()
        st = load().logo_server_create(ctypes.byref(o), ctypes.byref(h))
        if st:
            raise LogoError(st, load().logo_server_last_error(None).decode(errors="replace"))
        self._h = h
        self._n = {}

    def close(self):
        if getattr(self, "_h", None):
            load().logo_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _err(self, st):
        raise LogoError(st, load().logo_server_last_error(self._h).decode(errors="replace"))

    def submit(self, coords, route, seed):
        xy = np.ascontiguousarray(coords, dtype=np.float32).reshape(-1, 2)
        r = np.ascontiguousarray(route, dtype=np.uint32)
        rid = ctypes.c_uint64()
        st = load().logo_server_submit(self._h, xy.ctypes.data, len(r), r.ctypes.data_as(_u32p),
                                       int(seed) & ((1 << 64) - 1), ctypes.byref(rid))
        if st:
            self._err(st)
        self._n[rid.value] = len(r)
        return rid.value

    def _result(self, st, rid, out, info):
        if st == self.BUSY:
            return None
        self._n.pop(rid, None)
        d = {k: getattr(info, k) for k, _ in RequestInfo._fields_}
        if st:
            d["error"] = STATUS.get(st, st)
            return None, d
        return out, d

    def poll(self, rid):
        """None while running, else (route, info)."""
        out = np.zeros(self._n[rid], dtype=np.uint32)
        info = RequestInfo()
        st = load().logo_server_poll(self._h, rid, out.ctypes.data_as(_u32p), ctypes.byref(info))
        return self._result(st, rid, out, info)

    def wait(self, rid, timeout_ms=600000):
        out = np.zeros(self._n[rid], dtype=np.uint32)
        info = RequestInfo()
        st = load().logo_server_wait(self._h, rid, timeout_ms, out.ctypes.data_as(_u32p),
                                     ctypes.byref(info))
        return self._result(st, rid, out, info)

    def stats(self):
        s = ServerStats()
        st = load().logo_server_get_stats(self._h, ctypes.byref(s))
        if st:
            self._err(st)
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}
