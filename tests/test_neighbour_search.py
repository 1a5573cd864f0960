"""Neighbour lists and the neighbour-list search, on the CPU.

* logo_neighbours (the library's grid search, csrc/construct.cpp) equals the
  oracle's brute-force lists exactly: uniform and clustered binary32
  instances, an integer grid with many equal distances and duplicate points,
  tours of 1 to 20 cities (fewer other cities than list slots), a single
  repeated point, and the longest list.
* The oracle's neighbour search is pinned to the reference-pinned full
  search: with lists of every other city (k = n - 1) its candidate pairs are
  all pairs of the sweep, so the descent must be move for move the oracle's
  exhaustive one; with short lists it must still end at a 2-opt local
  optimum (no improving pair at all) with a valid tour.
"""
import numpy as np
import pytest


def _instances(inst):
    yield inst.uniform_f32(3000, 1, 1.0e6)
    yield inst.clustered(4000, 2, side=1.0e6, clusters=20)
    yield np.floor(inst.uniform_int(2500, 3) / 50.0).astype(np.float32)
    yield np.full((12, 2), 7.5, dtype=np.float32)


@pytest.mark.parametrize("k", [1, 5, 8, 16])
def test_library_lists_equal_the_oracle(lg, inst, oracle_mod, k):
    for xy in _instances(inst):
        assert np.array_equal(lg.neighbours(xy, k), oracle_mod.knn(xy, k)), (len(xy), k)


def test_threaded_lists_equal_the_oracle(lg, inst, oracle_mod):
    """From 20,000 cities the library splits the cities over host threads;
    the lists must not depend on it."""
    xy = inst.clustered(24000, 8, side=1.0e6, clusters=30)
    assert np.array_equal(lg.neighbours(xy, 8), oracle_mod.knn(xy, 8))
    xy = np.floor(inst.uniform_int(21000, 9) / 50.0).astype(np.float32)
    assert np.array_equal(lg.neighbours(xy, 5), oracle_mod.knn(xy, 5))


def test_small_and_longest_lists(lg, inst, oracle_mod):
    for n in range(1, 21):
        xy = inst.uniform_int(n, 100 + n)
        for k in (1, 3, 16, 64):
            assert np.array_equal(lg.neighbours(xy, k), oracle_mod.knn(xy, k)), (n, k)
    with pytest.raises(lg.LogoError):
        lg.neighbours(inst.uniform_int(10, 1), 65)


def test_full_lists_give_the_exhaustive_descent(inst, oracle_mod):
    for n, seed in ((17, 1), (12, 2), (9, 3)):
        for xy in (inst.uniform_int(n, seed), inst.uniform_f32(n, seed, 100.0)):
            r = inst.random_tour(n, seed)
            want, m, _ = oracle_mod.descend(xy, r)
            got, m2, nm = oracle_mod.descend_nbr(xy, r, k=n - 1)
            assert np.array_equal(got, want) and m2 == m and nm == m


def test_short_lists_end_at_a_local_optimum(inst, oracle_mod):
    for xy, r in ((inst.uniform_f32(1500, 4, 1.0e4), inst.random_tour(1500, 4)),
                  (inst.clustered(1200, 5, side=1.0e6, clusters=8), None)):
        if r is None:
            r = np.arange(len(xy), dtype=np.uint32)
        got, m, nm = oracle_mod.descend_nbr(xy, r, k=5, threads=4)
        assert oracle_mod.check_tour(got, len(xy))
        assert oracle_mod.best_move(xy, got) == (0, 0, 0)
        assert 0 < nm <= m
        assert oracle_mod.tour_length(xy, got) < oracle_mod.tour_length(xy, r)


def test_oropt_steps_change_the_length_by_their_delta(inst, oracle_mod):
    """Every step of the search with Or-opt moves changes the tour length by
    exactly the delta it was chosen with, keeps a permutation, and Or-opt
    moves of every variant (segment lengths 1-3, in order and reversed,
    moved left and right) occur."""
    seen = set()
    for n, seed in ((400, 1), (250, 2), (120, 3)):
        xy = inst.uniform_f32(n, seed, 1.0e4)
        r = inst.random_tour(n, seed)
        nb = oracle_mod.knn(xy, 8)
        for _ in range(400):
            step = oracle_mod.nbr_step(xy, r, 8, oropt=True, nb=nb)
            if step is None:
                break
            d, slot, i, j = step
            before = oracle_mod.tour_length(xy, r)
            r2, m, _ = oracle_mod.descend_nbr(xy, r, 8, max_moves=1, stop_at_limit=True,
                                              oropt=True)
            assert m == 1 and oracle_mod.check_tour(r2, n)
            assert oracle_mod.tour_length(xy, r2) - before == d < 0
            if slot >= 0:
                seen.add((slot, j > i))
            r = r2
    assert {s for s, _ in seen} == {0, 1, 2, 3, 4}
    assert {right for _, right in seen} == {False, True}


def test_oropt_search_ends_at_a_local_optimum(inst, oracle_mod):
    for xy, r in ((inst.uniform_f32(1500, 6, 1.0e4), inst.random_tour(1500, 6)),
                  (inst.clustered(1200, 7, side=1.0e6, clusters=8), None)):
        if r is None:
            r = np.arange(len(xy), dtype=np.uint32)
        got, m, nm = oracle_mod.descend_nbr(xy, r, k=8, threads=4, oropt=True)
        plain, _, _ = oracle_mod.descend_nbr(xy, r, k=8, threads=4)
        assert oracle_mod.check_tour(got, len(xy))
        assert oracle_mod.best_move(xy, got) == (0, 0, 0)
        assert 0 < nm <= m
        assert oracle_mod.tour_length(xy, got) < oracle_mod.tour_length(xy, plain)


def test_host_builders_do_not_depend_on_the_thread_count(lg, inst, monkeypatch):
    """The multiple-fragment tour and the neighbour lists split their
    per-city queries over host threads from 20,000 cities; one thread gives
    the same result."""
    xy = inst.clustered(30000, 11, side=1.0e6, clusters=60)
    dup = np.floor(inst.uniform_int(22000, 12) / 40.0).astype(np.float32)
    many = (lg.mf_tour(xy), lg.mf_tour(dup), lg.neighbours(xy, 8), lg.neighbours(dup, 6))
    monkeypatch.setenv("LOGO_HOST_THREADS", "1")
    one = (lg.mf_tour(xy), lg.mf_tour(dup), lg.neighbours(xy, 8), lg.neighbours(dup, 6))
    monkeypatch.setenv("LOGO_HOST_THREADS", "3")
    three = (lg.mf_tour(xy), lg.mf_tour(dup), lg.neighbours(xy, 8), lg.neighbours(dup, 6))
    for a, b, c in zip(many, one, three):
        assert np.array_equal(a, b) and np.array_equal(a, c)
    assert lg.check_tour(many[0]) and lg.check_tour(many[1])
