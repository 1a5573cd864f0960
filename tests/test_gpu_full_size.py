"""Parity at the sizes the benchmark and the workload configurations run.

Each test compares the sm_103a path with the CPU oracle (itself pinned to the
reference's own code) on the full-size inputs, using the oracle's threaded
sweep so that a 5e9-pair sweep takes well under a second of host time:

* states along the whole n = 100,000 descent that bench.py times (Gaussian
  mixture, nearest-neighbour start): the start, every 500th move, the last
  five moves and the local optimum;
* one sweep of n = 1,000,000 uniform points on a random tour (the largest
  sweep-throughput case, about 5e11 pairs);
* a reduced large-instance run (n = 20,000 Gaussian mixture, nearest-neighbour
  start, descent + 20 double-bridge kicks through logo_ils) against the
  oracle's ILS: best tour, length, moves and acceptances;
* the neighbour-list search (LOGO_SEARCH_NEIGHBOUR, 8 nearest cities) on a
  25,000-city Gaussian mixture from its nearest-neighbour tour (the boxed
  screen finishes the descent): the whole descent against the oracle's
  restatement (tour, moves, length).  At the benchmark's 100,000 cities the
  oracle needs about 700 full sweeps after the neighbour phase, several
  minutes of host time.

The reference loop these follow is CPUSolver::optimizeStep
(src/solvers/cpuSolver.cpp:104-146) inside TwoOptLocalSolver::optimize
(src/solvers/twoOptLocalSolver.cpp:22-64) and ILSGlobalSolverSequential::optimize
(src/solvers/ILSGlobalSolverSequential.cpp:60-100).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def _oracle_move(oracle, xy, route):
    key = oracle.best_move_key(xy, route, threads=THREADS)
    if key == (1 << 64) - 1:
        return (0, 0, 0)
    return oracle.unpack_key(key)


def test_states_along_the_benchmark_descent(lg, inst, oracle_mod):
    n = 100000
    xy = inst.clustered(n, 2, side=1.0e6, clusters=200, sigma_frac=0.01)
    r0 = lg.nn_tour(xy, 0)
    with lg.Solver(xy) as s:
        final, st = s.optimize(r0)
        m = st["moves"]
        assert m > 10000  # the benchmark's descent: about 14,500 moves
        ks = sorted(set(range(0, m - 5, 500)) | {m - 5, m - 4, m - 3, m - 2, m - 1, m})
        s.set_route(r0)
        done = 0
        checked = 0
        for k in ks:
            if k > done:
                got_moves = s.descend_resident(k - done)["moves"]
                assert got_moves == k - done, (k, got_moves)
                done = k
            r = s.get_route()
            want = _oracle_move(oracle_mod, xy, r)
            assert s.sweep_resident() == want, k
            checked += 1
        assert np.array_equal(s.get_route(), final)
        assert want == (0, 0, 0)  # the local optimum has no improving move
    assert checked >= 30


def test_million_city_sweep(lg, inst, oracle_mod):
    n = 1000000
    xy = inst.uniform_f32(n, 4, 1.0e6)
    r = inst.random_tour(n, 4)
    with lg.Solver(xy) as s:
        got = s.optimize_step(r)
    assert got == _oracle_move(oracle_mod, xy, r)


def test_reduced_large_instance_ils(lg, inst, oracle_mod):
    n = 20000
    xy = inst.clustered(n, 6, side=1.0e6, clusters=200, sigma_frac=0.01)
    r0 = lg.nn_tour(xy, 0)
    want, wst = oracle_mod.ils(xy, r0, 20, 77, oracle_mod.KICK_DOUBLE_BRIDGE, threads=THREADS)
    with lg.Solver(xy) as s:
        got, st = s.ils(r0, 20, 77, lg.KICK_DOUBLE_BRIDGE)
    assert st["final_length"] == wst["best_length"]
    assert st["moves"] == wst["moves"] and st["accepted"] == wst["accepted"]
    assert np.array_equal(got, want)


def test_neighbour_search_descent_on_a_boxed_size_instance(lg, inst, oracle_mod):
    n = 25000
    xy = inst.clustered(n, 12, side=1.0e6, clusters=50, sigma_frac=0.01)
    r0 = lg.nn_tour(xy, 0)
    want, m, nm = oracle_mod.descend_nbr(xy, r0, k=8, threads=THREADS)
    with lg.Solver(xy) as s:
        assert s.info()["variant"] == lg.SWEEP_BOXED
        s.set_search(lg.SEARCH_NEIGHBOUR, 8)
        got, st = s.optimize(r0)
    assert st["moves"] == m and nm > 2500 and m > nm
    assert st["final_length"] == oracle_mod.tour_length(xy, want)
    assert np.array_equal(got, want)
