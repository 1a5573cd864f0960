"""Seeded generators: determinism, ranges and the SplitMix64 stream shared
with the oracle and the device.  CPU only."""
import numpy as np


def test_splitmix_matches_oracle(inst, oracle_mod):
    a = inst.splitmix64(12345, 8)
    b = oracle_mod.splitmix_sequence(12345, 8)
    assert [int(x) for x in a] == b
    s = 12345
    for v in b:
        o, s = inst.splitmix64_scalar(s)
        assert o == v


def test_generators_are_deterministic_and_in_range(inst):
    a = inst.uniform_int(1000, 1)
    assert np.array_equal(a, inst.uniform_int(1000, 1))
    assert a.dtype == np.float32 and a.min() >= 0 and a.max() <= 9999
    assert np.all(a == np.floor(a))
    b = inst.uniform_f32(5000, 2, 1.0e6)
    assert b.min() >= 0 and b.max() < 1.0e6
    c = inst.clustered(20000, 3)
    assert c.min() >= 0 and c.max() < 1.0e6
    # 200 clusters with sigma 1e4: most points lie within 4 sigma of a centre
    assert not np.array_equal(c, inst.clustered(20000, 4))


def test_pinned_values(inst):
    """First values of each generator, so that a change to a generator is a
    deliberate, visible edit (the golden fixtures also hash instances)."""
    assert inst.uniform_int(3, 1).tolist() == [[5976.0, 2917.0], [4904.0, 8455.0],
                                               [9721.0, 1090.0]]
    assert inst.uniform_f32(2, 1, 1e6).tolist() == [[37631.75, 974481.5625],
                                                    [664787.9375, 717290.3125]]
    assert inst.clustered(2, 1).tolist() == [[256045.46875, 743755.1875],
                                             [799165.75, 860180.5]]
    assert inst.random_tour(10, 1).tolist() == [7, 8, 6, 0, 3, 5, 2, 4, 9, 1]
    assert inst.batch_sizes(5, 1).tolist() == [890, 422, 373, 210, 785]


def test_random_tour_is_a_permutation(inst, oracle_mod):
    for n in (3, 10, 1001):
        t = inst.random_tour(n, n)
        assert oracle_mod.check_tour(t)


def test_batched_workload_shape(inst):
    ns = inst.batch_sizes(4096, 5)
    assert ns.min() >= 50 and ns.max() <= 2000
    # log-uniform: the median sits near sqrt(50*2000) = 316
    assert 250 < np.median(ns) < 400
    coords, routes, seeds = inst.batched_workload(8, 5)
    assert len(coords) == 8 and all(len(c) == len(r) for c, r in zip(coords, routes))
    assert len(set(seeds)) == 8
