"""The neighbour-list search (LOGO_SEARCH_NEIGHBOUR) on the device against
the oracle's restatement of it (oracle/oracle.c, lo_descend_nbr / lo_ils_nbr,
whose candidate enumeration is pinned to the exhaustive oracle by
tests/test_neighbour_search.py).

* Descents: final tour, move count and the neighbour phase's moves equal
  the oracle's, on uniform, clustered and integer-grid instances (equal
  distances, duplicate points), from random and nearest-neighbour tours,
  with the MUFU screen (n = 1000, 5000) and the boxed screen (n = 24,000,
  nearest-neighbour starts) finishing the descent, and with lists of 4, 5,
  8 and 16 cities.
* With lists of every other city (n = 17, k = 16) the search is the
  reference's exhaustive descent, move for move.
* A move limit stops the search where the oracle's stops.
* ILS in neighbour mode (segment and double-bridge kicks, the device-run
  ILS graph) equals the oracle's ILS with the same descents.
* Switching a context back to the exhaustive search gives the reference's
  descent again.
* The same with Or-opt candidates (LOGO_SEARCH_NEIGHBOUR_OROPT, oracle
  lo_descend_nbr / lo_ils_nbr with oropt): descents, a move limit and ILS.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def _case(lg, inst, kind, n, seed):
    if kind == "uniform":
        xy = inst.uniform_f32(n, seed, 1.0e6)
    elif kind == "clustered":
        xy = inst.clustered(n, seed, side=1.0e6, clusters=max(2, n // 250))
    else:
        xy = np.floor(inst.uniform_int(n, seed) / 40.0).astype(np.float32)
    r = inst.random_tour(n, seed) if seed % 2 else lg.nn_tour(xy, 0)
    return xy, r


@pytest.mark.parametrize("kind,n,seed,k,oropt", [
    ("uniform", 1000, 1, 8, False), ("clustered", 1000, 2, 4, False), ("grid", 1000, 3, 16, False),
    ("uniform", 5000, 4, 8, False), ("grid", 5000, 5, 8, False), ("clustered", 24000, 6, 8, False),
    ("uniform", 24000, 8, 8, False),
    ("uniform", 1000, 1, 8, True), ("grid", 1000, 3, 5, True), ("clustered", 5000, 8, 8, True),
    ("grid", 3000, 9, 16, True), ("uniform", 12000, 10, 8, True),
])
def test_descent_matches_the_oracle(lg, inst, oracle_mod, kind, n, seed, k, oropt):
    xy, r = _case(lg, inst, kind, n, seed)
    want, m, nm = oracle_mod.descend_nbr(xy, r, k=k, threads=THREADS, oropt=oropt)
    mode = lg.SEARCH_NEIGHBOUR_OROPT if oropt else lg.SEARCH_NEIGHBOUR
    with lg.Solver(xy) as s:
        s.set_search(mode, k)
        info = s.info()
        assert info["search"] == mode and info["search_neighbours"] == k
        got, st = s.optimize(r)
        assert st["moves"] == m
        assert st["final_length"] == oracle_mod.tour_length(xy, want)
        assert np.array_equal(got, want)
        # fewer pairs than full sweeps would decide
        assert st["pair_evals"] < st["sweeps"] * (n - 2) * (n - 3) // 2
        # the same from a resident tour, and with the C-ABI in place
        s.set_route(r)
        assert s.descend_resident()["moves"] == m
        assert np.array_equal(s.get_route(), want)
        buf = r.copy()
        s.optimize_inplace(buf)
        assert np.array_equal(buf, want)
    assert nm > 0


def test_full_lists_are_the_exhaustive_descent(lg, inst, oracle_mod):
    n = 17
    for seed in range(4):
        xy = inst.uniform_int(n, 60 + seed)
        r = inst.random_tour(n, 60 + seed)
        want, m, _ = oracle_mod.descend(xy, r)
        with lg.Solver(xy) as s:
            s.set_search(lg.SEARCH_NEIGHBOUR, 16)
            got, st = s.optimize(r)
        assert np.array_equal(got, want) and st["moves"] == m


@pytest.mark.parametrize("limit,oropt", [(1, False), (7, False), (40, False), (1, True),
                                         (33, True)])
def test_move_limit(lg, inst, oracle_mod, limit, oropt):
    xy, r = _case(lg, inst, "uniform", 3000, 11)
    want, m, _ = oracle_mod.descend_nbr(xy, r, k=8, max_moves=limit, threads=THREADS,
                                       stop_at_limit=True, oropt=oropt)
    with lg.Solver(xy) as s:
        s.set_search(lg.SEARCH_NEIGHBOUR_OROPT if oropt else lg.SEARCH_NEIGHBOUR)
        got, st = s.optimize(r, max_moves=limit)
    assert st["moves"] == m == limit
    assert np.array_equal(got, want)


@pytest.mark.parametrize("n,kicks,kind,oropt", [(2000, 12, 1, False), (3000, 8, 0, False),
                                                (20000, 4, 1, False), (2000, 12, 1, True),
                                                (8000, 4, 0, True)])
def test_ils_matches_the_oracle(lg, inst, oracle_mod, n, kicks, kind, oropt):
    xy, r = _case(lg, inst, "clustered", n, 20 + n)
    want, wst = oracle_mod.ils_nbr(xy, r, kicks, 5, kind, k=8, threads=THREADS, oropt=oropt)
    with lg.Solver(xy) as s:
        s.set_search(lg.SEARCH_NEIGHBOUR_OROPT if oropt else lg.SEARCH_NEIGHBOUR)
        got, st = s.ils(r, kicks, 5, kind)
    assert st["final_length"] == wst["best_length"]
    assert st["moves"] == wst["moves"] and st["accepted"] == wst["accepted"]
    assert np.array_equal(got, want)


def test_switching_back_to_the_exhaustive_search(lg, inst, oracle_mod):
    xy, r = _case(lg, inst, "uniform", 2500, 31)
    want, m, _ = oracle_mod.descend(xy, r, threads=THREADS)
    with lg.Solver(xy) as s:
        s.set_search(lg.SEARCH_NEIGHBOUR, 6)
        s.optimize(r)
        s.set_search(lg.SEARCH_EXHAUSTIVE)
        got, st = s.optimize(r)
        assert s.info()["descent_mode"] == lg.DESCENT_COOPERATIVE
    assert np.array_equal(got, want) and st["moves"] == m
    with lg.Solver(xy) as s, pytest.raises(lg.LogoError):
        s.set_search(lg.SEARCH_NEIGHBOUR, 17)


def test_tiny_tours_in_both_neighbour_modes(lg, inst, oracle_mod):
    """3 to 12 cities (fewer other cities than list slots, segments that do
    not fit): descents and a short ILS equal the oracle's in both modes."""
    for n in range(3, 13):
        for seed in (1, 2):
            xy = inst.uniform_int(n, 300 + 10 * n + seed)
            r = inst.random_tour(n, 400 + 10 * n + seed)
            for oropt in (False, True):
                want, m, _ = oracle_mod.descend_nbr(xy, r, k=8, oropt=oropt)
                wils, wst = oracle_mod.ils_nbr(xy, r, 5, 3, 1, k=8, oropt=oropt)
                with lg.Solver(xy) as s:
                    s.set_search(lg.SEARCH_NEIGHBOUR_OROPT if oropt else lg.SEARCH_NEIGHBOUR)
                    got, st = s.optimize(r)
                    gils, gst = s.ils(r, 5, 3, lg.KICK_DOUBLE_BRIDGE)
                assert np.array_equal(got, want) and st["moves"] == m, (n, oropt)
                assert np.array_equal(gils, wils) and gst["final_length"] == wst["best_length"]


@pytest.mark.parametrize("n,oropt", [(700, False), (9000, False), (30000, False), (4000, True),
                                     (20000, True)])
def test_cooperative_and_graph_neighbour_phase_agree(lg, inst, n, oropt):
    """The neighbour phase as one cooperative launch (the default) and as
    graph launches (LOGO_DESCENT_GRAPH) give the same tour, moves and
    statistics."""
    xy, r = _case(lg, inst, "clustered", n, 50 + n)
    runs = []
    for mode in (lg.DESCENT_AUTO, lg.DESCENT_GRAPH):
        with lg.Solver(xy) as s:
            s.set_search(lg.SEARCH_NEIGHBOUR_OROPT if oropt else lg.SEARCH_NEIGHBOUR)
            s.set_descent_mode(mode)
            got, st = s.optimize(r)
            limited, st2 = s.optimize(r, max_moves=37)
        runs.append((got, st["moves"], st["sweeps"], st["pair_evals"], st["final_length"],
                     limited, st2["moves"]))
    a, b = runs
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[5], b[5])
    assert a[1:5] == b[1:5] and a[6] == b[6] == 37
