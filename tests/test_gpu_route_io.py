"""Route transfer modes of the single-instance context.

LOGO_ROUTE_IO_DIRECT lets the load and store kernels read and write the
caller's route buffer in place (where the device reaches pageable host
memory); LOGO_ROUTE_IO_COPY copies it with cudaMemcpyAsync.  Every entry
point that takes or returns a route must give the same results in both
modes, and the same as the oracle: logo_best_move, logo_tour_length,
logo_descend (one move, a few moves, to the local optimum, with and without
stats), logo_ils, logo_set_route / logo_get_route around a resident descent,
and a bad route followed by a good one.  Sizes cover the cooperative descent
(n = 700), the graph descent with the MUFU screen (n = 3001) and the boxed
screen (n = 30,000).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def _modes(lg, xy):
    modes = [lg.ROUTE_IO_COPY]
    with lg.Solver(xy) as s:
        try:
            s.set_route_io(lg.ROUTE_IO_DIRECT)
            modes.append(lg.ROUTE_IO_DIRECT)
        except lg.LogoError:
            pass
    return modes


def _oracle_moves(oracle, xy, r, k):
    r = np.array(r, dtype=np.uint32, copy=True)
    m = 0
    for _ in range(k):
        key = oracle.best_move_key(xy, r, threads=THREADS)
        if key == (1 << 64) - 1:
            break
        _, i, j = oracle.unpack_key(key)
        r = oracle.apply_move(r, i, j)
        m += 1
    return r, m


def _run_all(lg, xy, r, mode):
    out = {}
    with lg.Solver(xy) as s:
        s.set_route_io(mode)
        assert s.info()["route_io"] == mode
        out["move"] = s.optimize_step(r)
        out["length"] = s.route_length(r)
        one = r.copy()
        assert s.optimize_inplace(one, max_moves=1) is None
        out["one"] = one
        five = r.copy()
        st5 = s.optimize_inplace(five, max_moves=5, stats=True)
        out["five"] = (five, st5["moves"], st5["final_length"])
        full, st = s.optimize(r, stats=False)
        out["full"] = full
        full2, st2 = s.optimize(r)
        assert np.array_equal(full, full2)
        out["full_stats"] = (st2["moves"], st2["start_length"], st2["final_length"])
        best, sti = s.ils(r, 6, 11, lg.KICK_DOUBLE_BRIDGE)
        out["ils"] = (best, sti["final_length"], sti["moves"], sti["accepted"])
        s.set_route(r)
        s.descend_resident(3)
        out["resident"] = s.get_route()
        bad = r.copy()
        bad[5] = bad[6]
        with pytest.raises(lg.LogoError) as e:
            s.optimize_inplace(bad, max_moves=1)
        assert e.value.status == 1
        out["after_bad"] = s.optimize_step(r)
    return out


@pytest.mark.parametrize("n", [700, 3001, 30000])
def test_route_modes_agree_with_each_other_and_the_oracle(lg, inst, oracle_mod, n):
    xy = inst.clustered(n, 40 + n, side=1.0e6, clusters=max(2, n // 300))
    r = inst.random_tour(n, 41 + n) if n < 10000 else lg.nn_tour(xy, 0)
    runs = {m: _run_all(lg, xy, r, m) for m in _modes(lg, xy)}
    first = runs[lg.ROUTE_IO_COPY]
    for m, got in runs.items():
        for k, v in first.items():
            if isinstance(v, tuple):
                assert all(np.array_equal(a, b) for a, b in zip(v, got[k])), (m, k)
            else:
                assert np.array_equal(v, got[k]), (m, k)
    key = oracle_mod.best_move_key(xy, r, threads=THREADS)
    want = (0, 0, 0) if key == (1 << 64) - 1 else oracle_mod.unpack_key(key)
    assert first["move"] == want and first["after_bad"] == want
    assert first["length"] == oracle_mod.tour_length(xy, r)
    w1, _ = _oracle_moves(oracle_mod, xy, r, 1)
    assert np.array_equal(first["one"], w1)
    w5, m5 = _oracle_moves(oracle_mod, xy, r, 5)
    assert np.array_equal(first["five"][0], w5) and first["five"][1] == m5
    assert first["five"][2] == oracle_mod.tour_length(xy, w5)
    if n <= 3001:
        wf, mf, _ = oracle_mod.descend(xy, r, threads=THREADS)
        assert np.array_equal(first["full"], wf) and first["full_stats"][0] == mf


def test_direct_mode_reads_the_buffer_each_call(lg, inst):
    """The device reads the caller's buffer at the time of each call (no
    stale copy): a buffer rewritten between calls gives the new answer."""
    n = 2000
    xy = inst.uniform_f32(n, 9, 1.0e4)
    if lg.ROUTE_IO_DIRECT not in _modes(lg, xy):
        pytest.skip("the device cannot reach pageable host memory")
    a, b = inst.random_tour(n, 1), inst.random_tour(n, 2)
    buf = a.copy()
    with lg.Solver(xy) as s, lg.Solver(xy) as ref:
        s.set_route_io(lg.ROUTE_IO_DIRECT)
        ref.set_route_io(lg.ROUTE_IO_COPY)
        assert s.optimize_step(buf) == ref.optimize_step(a)
        buf[:] = b
        assert s.optimize_step(buf) == ref.optimize_step(b)
        buf[:] = a
        s.optimize_inplace(buf, max_moves=2)
        want = a.copy()
        ref.optimize_inplace(want, max_moves=2)
        assert np.array_equal(buf, want)
