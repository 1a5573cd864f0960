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
