"""Parity of the sm_103a path with the CPU oracle, through the C ABI.

The bar is bit-exactness: every (minchange, i, j), every tour and every length
must equal the oracle's, which is itself pinned to the reference's own code
(tests/test_oracle_ref.py, tests/test_oracle_golden.py).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [4, 5, 6, 7, 8, 9, 13, 31, 50, 64, 65, 100, 257, 500, 1000, 2000, 3001, 5000, 12001]


def _instance(inst, n, seed):
    kind = seed % 3
    if kind == 0:
        return inst.uniform_int(n, seed)
    if kind == 1:
        return inst.uniform_f32(n, seed, 1.0e4)
    return inst.clustered(n, seed, side=1.0e6, clusters=max(2, n // 50))


def _replay(oracle, route, log, k):
    r = np.array(route, dtype=np.uint32)
    for d, i, j in log[:k]:
        r = oracle.apply_move(r, int(i), int(j))
    return r


@pytest.mark.parametrize("n", SIZES)
def test_best_move_matches_oracle(lg, inst, oracle_mod, n):
    seeds = range(3) if n > 3000 else range(8)
    for seed in seeds:
        xy = _instance(inst, n, seed)
        r = inst.random_tour(n, seed + 100)
        with lg.Solver(xy) as s:
            assert s.optimize_step(r) == oracle_mod.best_move(xy, r), (n, seed)


def test_small_tours_match_reference_fixture(lg, inst):
    """Tours of 4 to 7 cities from small_n.npz (written by the reference's
    own code): single step, whole descent and batched descent.  At n = 4 the
    one pair (1, 2) is evaluated and reported as (1, 3), as the reference's
    loop does."""
    import hashlib
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "small_n.npz"))
    square = np.array([[0, 0], [10, 0], [10, 10], [0, 10]], dtype=np.float32)
    cases = []
    for k, (gi, n, seed, rseed, m, length) in enumerate(g["spec"]):
        if gi < 0:
            xy, r = square, np.array([0, 2, 1, 3], dtype=np.uint32)
        else:
            xy = _instance_gen(inst, int(gi), int(n), int(seed))
            r = inst.random_tour(int(n), int(rseed))
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(xy).tobytes())
        h.update(np.ascontiguousarray(r).tobytes())
        assert h.hexdigest() == g["hash"][k]
        final = g["final"][g["final_offsets"][k]:g["final_offsets"][k + 1]]
        with lg.Solver(xy) as s:
            assert s.optimize_step(r) == tuple(int(v) for v in g["out"][k]), (n, seed)
            got, st = s.optimize(r)
        assert np.array_equal(got, final) and st["moves"] == m and st["final_length"] == length
        cases.append((xy, r, final, length))
    with lg.Batch(len(cases), sum(len(c[1]) for c in cases)) as b:
        got, res, _ = b.solve([c[0] for c in cases], [c[1] for c in cases],
                              list(range(len(cases))), kicks=0)
    for k, (xy, r, final, length) in enumerate(cases):
        assert res[k]["best_length"] == length and np.array_equal(got[k], final), k


def _instance_gen(inst, gi, n, seed):
    if gi == 0:
        return inst.uniform_int(n, seed)
    if gi == 1:
        return inst.uniform_f32(n, seed, 1.0e4)
    return inst.clustered(n, seed, side=1.0e6, clusters=max(2, n // 50))


@pytest.mark.parametrize("n", [60, 300, 1000])
def test_best_move_near_local_optimum(lg, inst, oracle_mod, n):
    """States late in a descent: small deltas and many ties."""
    xy = inst.uniform_int(n, 7)
    r0 = inst.random_tour(n, 7)
    _, m, log = oracle_mod.descend(xy, r0, log_cap=1 << 20)
    with lg.Solver(xy) as s:
        for k in sorted({max(0, m - t) for t in (1, 2, 3, 5, 10, 30)} | {m}):
            r = _replay(oracle_mod, r0, log, k)
            assert s.optimize_step(r) == oracle_mod.best_move(xy, r), (n, k)


KERNELS = [(0, 2, 2, 64), (0, 2, 4, 32), (0, 4, 2, 128), (0, 4, 4, 64), (0, 4, 8, 256),
           (0, 8, 4, 1024), (0, 8, 8, 128), (0, 16, 4, 512),
           (4, 4, 2, 64), (4, 4, 4, 64), (4, 4, 8, 256), (4, 8, 2, 128), (4, 8, 4, 512),
           (4, 8, 8, 100), (4, 16, 4, 1024),
           (5, 4, 2, 64), (5, 4, 4, 64), (5, 4, 8, 256), (5, 8, 4, 512), (5, 8, 8, 100),
           (5, 16, 4, 1024),
           (6, 4, 2, 64), (6, 4, 4, 64), (6, 4, 8, 256), (6, 8, 4, 512), (6, 8, 8, 96),
           (6, 16, 4, 1024), (6, 4, 4, 32)]


@pytest.mark.parametrize("kernel", KERNELS)
def test_every_tile_shape(lg, inst, oracle_mod, kernel):
    """Every sweep variant (MUFU, fused, local and boxed screens) and every
    tile shape choose the oracle's move."""
    for n, seed in ((3001, 1), (777, 2), (70, 3)):
        xy = _instance(inst, n, seed)
        r = inst.random_tour(n, seed)
        with lg.Solver(xy) as s:
            s.set_kernel(*kernel)
            assert s.optimize_step(r) == oracle_mod.best_move(xy, r), (kernel, n)
            got, st = s.optimize(r, max_moves=25)
            want = r.copy()
            for _ in range(25):
                d, i, j = oracle_mod.best_move(xy, want)
                if d == 0:
                    break
                want = oracle_mod.apply_move(want, i, j)
            assert np.array_equal(got, want), kernel


VARIANTS = [(v, 8, 4, 128) for v in (0, 4, 5, 6)]


@pytest.mark.parametrize("kernel", VARIANTS)
def test_every_variant_near_local_optimum(lg, inst, oracle_mod, kernel):
    """Late-descent states of n = 3000 and 5000 tours (small deltas, tight
    screens): every variant chooses the oracle's move.  The states come from
    a device descent; only the single steps are compared."""
    for n, seed in ((3000, 11), (5000, 12)):
        xy = inst.clustered(n, seed, side=1.0e6, clusters=max(2, n // 500))
        r0 = inst.random_tour(n, seed)
        with lg.Solver(xy) as s:
            _, st = s.optimize(r0)
            m = st["moves"]
            states = [s.optimize(r0, max_moves=max(0, m - t))[0] for t in (0, 1, 3, 10, 100)]
        with lg.Solver(xy) as s:
            s.set_kernel(*kernel)
            for k, r in enumerate(states):
                assert s.optimize_step(r) == oracle_mod.best_move(xy, r), (kernel, n, k)


@pytest.mark.parametrize("mode", ["graph", "cooperative"])
@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_descent_move_sequence_plain_workload(lg, inst, oracle_mod, seed, mode):
    """n=1000 integer coordinates in [0,1e4)^2, random start: the whole move
    sequence, the final tour and its length equal the oracle's, with the
    graph-driven and the cooperative persistent descent."""
    xy = inst.uniform_int(1000, seed)
    r = inst.random_tour(1000, seed)
    want, m, log = oracle_mod.descend(xy, r, log_cap=1 << 20)
    with lg.Solver(xy) as s:
        s.set_descent_mode(lg.DESCENT_GRAPH if mode == "graph" else lg.DESCENT_COOPERATIVE)
        got, trace, st = s.optimize_trace(r)
    assert st["moves"] == m
    assert np.array_equal(trace, log)
    assert np.array_equal(got, want)
    assert st["final_length"] == oracle_mod.tour_length(xy, want)
    assert st["start_length"] == oracle_mod.tour_length(xy, r)
    assert st["sweeps"] == m + 1


@pytest.mark.parametrize("mode", ["graph", "cooperative"])
@pytest.mark.parametrize("n,kicks,kind", [(200, 40, 0), (200, 40, 1), (523, 25, 0),
                                          (523, 25, 1), (1500, 6, 1), (300, 0, 0),
                                          (3100, 8, 0), (3100, 8, 1)])
def test_ils_matches_oracle(lg, inst, oracle_mod, n, kicks, kind, mode):
    """The whole ILS call runs on the device: one cooperative launch, or one
    graph whose descent and kick loops are conditional WHILE nodes."""
    xy = inst.uniform_f32(n, n, 1.0e4)
    r = inst.random_tour(n, n + 1)
    want, ost = oracle_mod.ils(xy, r, kicks, 1234 + n, kind)
    with lg.Solver(xy) as s:
        s.set_descent_mode(lg.DESCENT_GRAPH if mode == "graph" else lg.DESCENT_COOPERATIVE)
        got, st = s.ils(r, kicks, 1234 + n, kind)
    assert np.array_equal(got, want)
    assert st["final_length"] == ost["best_length"]
    assert st["start_length"] == ost["start_length"]
    assert st["moves"] == ost["moves"]
    assert st["accepted"] == ost["accepted"]
    assert st["kicks"] == kicks


@pytest.mark.parametrize("mode", ["graph", "cooperative"])
def test_ils_waits_on_the_device_a_fixed_number_of_times(lg, inst, oracle_mod, mode):
    """An ILS call synchronises with the device a fixed number of times (the
    state read, the tour download, the timer), however many kicks it runs, on
    the cooperative launch and on the conditional graph."""
    n = 1200
    xy = inst.uniform_f32(n, 71, 1.0e4)
    r = inst.random_tour(n, 72)
    with lg.Solver(xy) as s:
        s.set_descent_mode(lg.DESCENT_GRAPH if mode == "graph" else lg.DESCENT_COOPERATIVE)
        waits = []
        for kicks in (2, 60):
            w0 = s.info()["host_waits"]
            got, st = s.ils(r, kicks, 5, lg.KICK_DOUBLE_BRIDGE)
            waits.append(s.info()["host_waits"] - w0)
            assert st["kicks"] == kicks
        want, ost = oracle_mod.ils(xy, r, 60, 5, lg.KICK_DOUBLE_BRIDGE,
                                   threads=os.cpu_count() or 4)
    assert np.array_equal(got, want) and st["final_length"] == ost["best_length"]
    assert waits[0] == waits[1] and waits[1] <= 4, waits


@pytest.mark.parametrize("n", [8, 2501, 6144])
def test_cooperative_descent_sizes(lg, inst, oracle_mod, n):
    """The cooperative descent at its size limits (smallest tour, the switch
    to 4-row tiles and 512-thread CTAs, the largest cooperative tour): bounded
    descents, traces and the resident tour agree with the graph-driven
    descent, whose moves are checked against the oracle elsewhere."""
    xy = inst.uniform_f32(n, 30 + n, 1.0e6)
    r = inst.random_tour(n, 31 + n)
    res = {}
    for mode in (lg.DESCENT_GRAPH, lg.DESCENT_COOPERATIVE):
        with lg.Solver(xy) as s:
            s.set_descent_mode(mode)
            assert s.info()["descent_mode"] == mode
            a, st_a = s.optimize(r, max_moves=7)
            b, tr, st_b = s.optimize_trace(a, max_moves=40)
            s.set_route(b)
            st_c = s.descend_resident(max_moves=0)
            res[mode] = (a, b, tr, s.get_route(), st_a["moves"], st_b["moves"], st_c["moves"],
                         st_c["sweeps"], s.length_resident())
    g, c = res[lg.DESCENT_GRAPH], res[lg.DESCENT_COOPERATIVE]
    for x, y in zip(g, c):
        if isinstance(x, np.ndarray):
            assert np.array_equal(x, y)
        else:
            assert x == y
    assert lg.check_tour(c[3])


def test_contexts_with_different_shared_memory_coexist(lg, inst, oracle_mod):
    """A kernel's shared-memory limit is one setting for the whole process: a
    context created later with a smaller tour or tile must not break the
    launches of one created earlier with a larger one."""
    big = inst.uniform_f32(6000, 41, 1.0e6)
    small = inst.uniform_f32(3000, 42, 1.0e6)
    rb, rs = inst.random_tour(6000, 43), inst.random_tour(3000, 44)
    with lg.Solver(big) as a:
        a.set_kernel(lg.SWEEP_LOCAL, 4, 4, 4096)
        with lg.Solver(small) as b:
            b.set_kernel(lg.SWEEP_LOCAL, 4, 4, 64)
            assert a.optimize_step(rb) == oracle_mod.best_move(big, rb)
            assert b.optimize_step(rs) == oracle_mod.best_move(small, rs)
            ta, sa = a.optimize(rb, max_moves=50)
            tb, sb = b.optimize(rs, max_moves=50)
            assert sa["moves"] == 50 and sb["moves"] == 50
            assert lg.check_tour(ta) and lg.check_tour(tb)


def test_descent_mode_api(lg, inst):
    xy = inst.uniform_f32(7000, 3, 1.0e6)
    with lg.Solver(xy) as s:
        assert s.info()["cooperative_ctas"] == 0
        assert s.info()["descent_mode"] == lg.DESCENT_GRAPH
        with pytest.raises(lg.LogoError):
            s.set_descent_mode(lg.DESCENT_COOPERATIVE)
        with pytest.raises(lg.LogoError):
            s.set_descent_mode(7)
    with lg.Solver(xy[:1000]) as s:
        assert s.info()["cooperative_ctas"] > 0
        assert s.info()["descent_mode"] == lg.DESCENT_COOPERATIVE


def test_tour_length_and_resident_api(lg, inst, oracle_mod):
    n = 4000
    xy = inst.uniform_f32(n, 5, 1.0e6)
    r = inst.random_tour(n, 5)
    with lg.Solver(xy) as s:
        assert s.route_length(r) == oracle_mod.tour_length(xy, r)
        s.set_route(r)
        assert np.array_equal(s.get_route(), r)
        assert s.sweep_resident() == oracle_mod.best_move(xy, r)
        st = s.descend_resident(max_moves=10)
        assert st["moves"] == 10
        want = r.copy()
        for _ in range(10):
            d, i, j = oracle_mod.best_move(xy, want)
            want = oracle_mod.apply_move(want, i, j)
        assert np.array_equal(s.get_route(), want)
        assert s.length_resident() == oracle_mod.tour_length(xy, want)


def test_degenerate_instances(lg, inst, oracle_mod):
    rng = np.random.default_rng(3)
    cases = []
    # duplicates and ties: integer grid far smaller than n
    cases.append(np.floor(rng.random((300, 2)) * 12).astype(np.float32))
    # all points identical (zero-length edges, no improving move)
    cases.append(np.full((50, 2), 7.0, dtype=np.float32))
    # collinear points
    cases.append(np.stack([np.arange(120, dtype=np.float32) * 3,
                           np.zeros(120, dtype=np.float32)], 1))
    # tiny and negative coordinates
    cases.append((rng.random((200, 2)).astype(np.float32) - 0.5) * 1e-3)
    for xy in cases:
        n = len(xy)
        r = inst.random_tour(n, n)
        want, m, log = oracle_mod.descend(xy, r, log_cap=1 << 20)
        with lg.Solver(xy) as s:
            assert s.optimize_step(r) == oracle_mod.best_move(xy, r)
            got, trace, st = s.optimize_trace(r)
        assert np.array_equal(trace, log)
        assert np.array_equal(got, want)


def test_three_and_four_city_tours(lg, inst, oracle_mod):
    """n = 3 has no pair; n = 4 has exactly one, (1, 2) reported as (1, 3),
    which the reference's loop evaluates (src/solvers/cpuSolver.cpp:104,123)."""
    xy = inst.uniform_int(3, 1)
    with lg.Solver(xy) as s:
        assert s.optimize_step(np.arange(3)) == (0, 0, 0)
        got, st = s.optimize(np.arange(3))
        assert st["moves"] == 0 and np.array_equal(got, np.arange(3))
    for seed in range(1, 6):
        xy = inst.uniform_int(4, seed)
        r = inst.random_tour(4, seed)
        with lg.Solver(xy) as s:
            assert s.optimize_step(r) == oracle_mod.best_move(xy, r), seed
            got, st = s.optimize(r)
        want, m, _ = oracle_mod.descend(xy, r)
        assert np.array_equal(got, want) and st["moves"] == m


def test_invalid_arguments(lg, inst):
    xy = inst.uniform_int(100, 1)
    with lg.Solver(xy) as s:
        bad = np.arange(100, dtype=np.uint32)
        bad[5] = 6
        with pytest.raises(lg.LogoError) as e:
            s.optimize_step(bad)
        assert e.value.status == 1
        bad = np.arange(100, dtype=np.uint32)
        bad[0] = 100
        with pytest.raises(lg.LogoError):
            s.optimize(bad)
    with pytest.raises(lg.LogoError):
        lg.Solver(xy[:2])
    nan = xy.copy()
    nan[3, 0] = np.nan
    with pytest.raises(lg.LogoError):
        lg.Solver(nan)
    far = xy.copy()
    far[0] = (3.0e6, 3.0e6)
    with pytest.raises(lg.LogoError):
        lg.Solver(far)


def test_bad_routes_rejected_then_context_usable(lg, inst, oracle_mod):
    """The route check runs on the device: a duplicate or out-of-range entry
    makes every entry point return INVALID_ARG, drops the resident route, and
    the next valid route works as usual."""
    n = 5000
    xy = inst.uniform_f32(n, 9, 1.0e6)
    r = inst.random_tour(n, 9)
    dup = r.copy()
    dup[n - 1] = dup[0]
    oor = r.copy()
    oor[1234] = n
    with lg.Solver(xy) as s:
        for bad in (dup, oor):
            for call in (s.optimize_step, s.optimize, s.route_length, s.set_route,
                         lambda b: s.ils(b, 2, 1, lg.KICK_SEGMENT)):
                with pytest.raises(lg.LogoError) as e:
                    call(bad)
                assert e.value.status == 1
            with pytest.raises(lg.LogoError):
                s.get_route()
        assert s.optimize_step(r) == oracle_mod.best_move(xy, r)
        assert s.route_length(r) == oracle_mod.tour_length(xy, r)
        got, st = s.optimize(r, max_moves=3)
        want = r.copy()
        for _ in range(3):
            d, i, j = oracle_mod.best_move(xy, want)
            want = oracle_mod.apply_move(want, i, j)
        assert np.array_equal(got, want) and st["moves"] == 3


def test_sqrt_error_bound(lg):
    """The filter margin assumes the approximate sqrt is within 2^-20
    relative; require 8x headroom over what the hardware actually does."""
    err = lg.sqrt_error(0)
    assert 0 < err <= 2.0 ** -23, err


def test_device_waits_give_up_then_context_usable(lg, inst, oracle_mod):
    """Failure detection without a fault: an mbarrier that expects bytes no
    copy delivers, and the cooperative grid barrier with one of its two CTAs
    missing, each give up after their 2 s budget and leave the timeout bit;
    the device then still solves correctly."""
    mbar, barrier, ms = lg.wait_limits(0)
    assert mbar == 1 and barrier == 1, (mbar, barrier)
    assert 3900.0 <= ms <= 30000.0, ms
    xy = _instance(inst, 300, 5)
    r = inst.random_tour(300, 105)
    with lg.Solver(xy) as s:
        assert s.optimize_step(r) == oracle_mod.best_move(xy, r)
        got, st = s.optimize(r, max_moves=5)
    want = r.copy()
    for _ in range(5):
        d, i, j = oracle_mod.best_move(xy, want)
        want = oracle_mod.apply_move(want, i, j)
    assert np.array_equal(got, want) and st["moves"] == 5


def test_timed_out_context_is_not_used_again(lg, inst, oracle_mod):
    """A device wait that gives up may leave a copy in flight, so its context
    refuses every later call.  The timeout bit is set by a test hook (no wait
    runs out here): the call that reads it returns TIMEOUT, every call after
    it DEVICE_FAULT, and a new context on the same device works."""
    xy = _instance(inst, 300, 6)
    r = inst.random_tour(300, 106)
    with lg.Solver(xy) as s:
        s.set_route(r)
        s.flag_timeout()
        with pytest.raises(lg.LogoError) as e:
            s.progress()
        assert e.value.status == 4
        for call in (lambda: s.optimize_step(r), lambda: s.optimize(r),
                     lambda: s.ils(r, 2, 1, lg.KICK_SEGMENT), lambda: s.route_length(r),
                     s.get_route, lambda: s.set_route(r), s.sweep_resident):
            with pytest.raises(lg.LogoError) as e:
                call()
            assert e.value.status == 5
    with lg.Solver(xy) as s:
        assert s.optimize_step(r) == oracle_mod.best_move(xy, r)


GROUPED_KERNELS = [(4, 4, 4, 256), (4, 4, 2, 256), (4, 4, 8, 128), (4, 8, 4, 512), (4, 8, 8, 256),
                   (4, 16, 4, 1024), (5, 4, 4, 256), (5, 4, 2, 256), (5, 4, 8, 128),
                   (5, 8, 4, 512), (5, 8, 8, 256), (5, 16, 4, 1024), (6, 4, 4, 256),
                   (6, 4, 2, 256), (6, 4, 8, 128), (6, 8, 4, 512), (6, 8, 8, 256),
                   (6, 16, 4, 1024), (6, 4, 4, 32)]


def test_grouped_paths_late_descent(lg, inst, oracle_mod):
    """n = 40,000 (the grouped column walks of the fused and local-coordinate
    screens): the NN start tour and states late in its descent (small deltas,
    tight screens) choose the oracle's move with every tile shape."""
    n = 40000
    xy = inst.clustered(n, 21, side=1.0e6, clusters=80, sigma_frac=0.01)
    r0, _ = oracle_mod.nn_tour(xy)
    threads = os.cpu_count() or 4
    with lg.Solver(xy) as s:
        _, st = s.optimize(r0)
        m = st["moves"]
        states = [r0] + [s.optimize(r0, max_moves=m - t)[0] for t in (0, 1, 4)]
    want = [oracle_mod.unpack_key(oracle_mod.best_move_key(xy, r, threads=threads))
            for r in states]
    assert want[1][0] == 0 and want[2][0] < 0
    with lg.Solver(xy) as s:
        for kernel in GROUPED_KERNELS:
            s.set_kernel(*kernel)
            for k, r in enumerate(states):
                assert s.optimize_step(r) == want[k], (kernel, k)


@pytest.mark.parametrize("n,gen,variant", [(100000, "clustered_nn", None),
                                           (100000, "clustered_nn", 4),
                                           (100000, "clustered_nn", 5),
                                           (100000, "clustered_nn", 6),
                                           (200000, "uniform_random", None),
                                           (200000, "uniform_random", 4),
                                           (200000, "uniform_random", 5),
                                           (200000, "uniform_random", 6)])
def test_large_sweep_matches_parallel_oracle(lg, inst, oracle_mod, n, gen, variant):
    """Full-size single sweeps against the oracle's multi-threaded sweep
    (default kernel and the square-root-free screens)."""
    if gen == "clustered_nn":
        xy = inst.clustered(n, 2)
        r, _ = oracle_mod.nn_tour(xy)
    else:
        xy = inst.uniform_f32(n, 3, 1.0e6)
        r = inst.random_tour(n, 3)
    threads = os.cpu_count() or 4
    key = oracle_mod.best_move_key(xy, r, threads=threads)
    with lg.Solver(xy) as s:
        if variant is not None:
            s.set_kernel(variant, 8, 4, 512)
        assert s.optimize_step(r) == oracle_mod.unpack_key(key)


@pytest.mark.parametrize("n,seed", [(30000, 41), (60000, 42)])
def test_full_descent_same_tour_every_large_variant(lg, inst, n, seed):
    """Whole descents from NN start tours at full size (thousands of sweeps,
    each late sweep with no improving move): the fused, local and boxed
    screens reach the same tour by the same number of moves as the MUFU
    screen, whose single steps are checked against the oracle above."""
    xy = inst.clustered(n, seed, side=1.0e6, clusters=n // 500, sigma_frac=0.01)
    r = lg.nn_tour(xy, 0)
    out = []
    for kernel in ((0, 4, 4, 128), (4, 4, 4, 512), (5, 4, 4, 512), (6, 4, 4, 512),
                   (6, 8, 8, 1024)):
        with lg.Solver(xy) as s:
            s.set_kernel(*kernel)
            got, st = s.optimize(r)
        out.append((kernel, got, st["moves"], st["final_length"]))
    for kernel, got, m, length in out[1:]:
        assert np.array_equal(got, out[0][1]), kernel
        assert (m, length) == (out[0][2], out[0][3]), kernel


@pytest.mark.parametrize("n,grid", [(3000, 8), (600, 3), (20000, 64)])
def test_boxed_seed_with_duplicate_points(lg, inst, oracle_mod, n, grid):
    """The boxed sweep seeds its bound from near-neighbour pairs; with many
    coincident cities (coordinates on a small integer grid) the neighbour
    lists are full of ties and zero distances.  Single steps and a short
    descent still equal the oracle's."""
    rng = np.random.default_rng(n)
    xy = (np.floor(rng.random((n, 2)) * grid) * 1000.0).astype(np.float32)
    r = inst.random_tour(n, n + 3)
    threads = os.cpu_count() or 4

    def move(route):
        key = oracle_mod.best_move_key(xy, route, threads=threads)
        return (0, 0, 0) if key == (1 << 64) - 1 else oracle_mod.unpack_key(key)

    with lg.Solver(xy) as s:
        s.set_kernel(lg.SWEEP_BOXED, 4, 4, 128)
        assert s.optimize_step(r) == move(r)
        got, st = s.optimize(r, max_moves=30)
    want = r.copy()
    for _ in range(30):
        d, i, j = move(want)
        if d == 0:
            break
        want = oracle_mod.apply_move(want, i, j)
    assert np.array_equal(got, want)


def test_retired_variants_rejected(lg, inst):
    """Variant numbers 1-3 are retired and refused; the context keeps working."""
    xy = inst.uniform_f32(300, 5, 1.0e4)
    r = inst.random_tour(300, 5)
    with lg.Solver(xy) as s:
        want = s.optimize_step(r)
        for v in (1, 2, 3, 7, -1):
            with pytest.raises(lg.LogoError) as e:
                s.set_kernel(v, 4, 4, 128)
            assert e.value.status == 1
        assert s.optimize_step(r) == want


def test_boxed_variant_tile_widths(lg, inst):
    """The boxed screen takes tile widths that are multiples of 32 up to 1024
    (one mask bit per 32-column window) and rejects the others."""
    xy = inst.uniform_f32(500, 3, 1.0e4)
    with lg.Solver(xy) as s:
        for cb in (100, 2048, 48):
            with pytest.raises(lg.LogoError) as e:
                s.set_kernel(lg.SWEEP_BOXED, 4, 4, cb)
            assert e.value.status == 1
        s.set_kernel(lg.SWEEP_BOXED, 4, 4, 1024)
        with pytest.raises(lg.LogoError):
            s.set_shape(4, 4, 1000)
        assert s.info()["variant"] == lg.SWEEP_BOXED and s.info()["tile_cols"] == 1024
