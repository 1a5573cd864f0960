"""Batched persistent solver: every instance must end exactly where the
oracle's ILS (and the single-instance GPU path) ends -- same best tour, same
best length, same move and acceptance counts."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload(inst, count, seed, n_lo=5, n_hi=400, extra=()):
    ns = list(inst.batch_sizes(count, seed, n_lo, n_hi)) + list(extra)
    coords, routes, seeds = [], [], []
    for k, n in enumerate(ns):
        s = inst.instance_seed(seed, k)
        coords.append(inst.uniform_f32(int(n), s, 1.0e4) if k % 3 else inst.uniform_int(int(n), s))
        routes.append(inst.random_tour(int(n), s))
        seeds.append(s)
    return coords, routes, seeds


@pytest.mark.parametrize("kind", [0, 1])
def test_batch_matches_oracle_ils(lg, inst, oracle_mod, kind):
    coords, routes, seeds = _workload(inst, 48, 11 + kind, extra=(3, 4, 5, 6))
    kicks = 12
    want_routes, want_len, want_moves = oracle_mod.ils_batch(coords, routes, seeds, kicks, kind,
                                                             threads=os.cpu_count() or 4)
    with lg.Batch(len(routes), sum(len(r) for r in routes)) as b:
        got, res, ms = b.solve(coords, routes, seeds, kicks=kicks, kind=kind)
    for k in range(len(routes)):
        assert res[k]["status"] == 0
        assert res[k]["best_length"] == want_len[k], k
        assert res[k]["moves"] == want_moves[k], k
        assert np.array_equal(got[k], want_routes[k]), k


def test_every_batch_shape_agrees(lg, inst, oracle_mod):
    coords, routes, seeds = _workload(inst, 24, 5, n_lo=20, n_hi=900)
    want_routes, want_len, _ = oracle_mod.ils_batch(coords, routes, seeds, 3, 0,
                                                    threads=os.cpu_count() or 4)
    shapes = [(2, 128, 64), (2, 256, 64), (4, 128, 64), (4, 256, 64), (4, 256, 128),
              (4, 512, 128), (8, 256, 128)]
    with lg.Batch(len(routes), sum(len(r) for r in routes)) as b:
        for sh in shapes:
            got, res, _ = b.solve(coords, routes, seeds, kicks=3, shape=sh)
            assert [r["best_length"] for r in res] == list(want_len), sh
            assert all(np.array_equal(g, w) for g, w in zip(got, want_routes)), sh


def test_batch_large_instances_match_single_instance_path(lg, inst):
    ns = [4096, 2500, 1999, 1024, 1023, 384, 383, 127]
    coords = [inst.uniform_f32(n, 100 + n, 1.0e4) for n in ns]
    routes = [inst.random_tour(n, 200 + n) for n in ns]
    seeds = [300 + n for n in ns]
    with lg.Batch(len(ns), sum(ns)) as b:
        got, res, _ = b.solve(coords, routes, seeds, kicks=2, kind=1)
    for k, n in enumerate(ns):
        with lg.Solver(coords[k]) as s:
            r, st = s.ils(routes[k], 2, seeds[k], 1)
        assert np.array_equal(got[k], r), n
        assert res[k]["best_length"] == st["final_length"], n
        assert res[k]["moves"] == st["moves"], n


def test_batch_autotune_keeps_results(lg, inst, tmp_path):
    coords, routes, seeds = _workload(inst, 40, 9, n_lo=30, n_hi=1500)
    cache = str(tmp_path / "tune.json")
    with lg.Batch(len(routes), sum(len(r) for r in routes)) as b:
        base, res0, _ = b.solve(coords, routes, seeds, kicks=2)
        b.autotune(coords, routes, seeds, kicks=2, cache_path=cache)
        tuned, res1, _ = b.solve(coords, routes, seeds, kicks=2)
        assert [r["best_length"] for r in res0] == [r["best_length"] for r in res1]
        assert all(np.array_equal(a, c) for a, c in zip(base, tuned))
        chosen = [b.shape_for(n) for n in (100, 300, 800, 1500)]
    text = open(cache).read()
    assert "|" in text and "[" in text
    with lg.Batch(len(routes), sum(len(r) for r in routes)) as b2:
        b2.autotune(coords, routes, seeds, kicks=2, cache_path=cache, reuse=True)
        assert [b2.shape_for(n) for n in (100, 300, 800, 1500)] == chosen


def test_batch_rejects_bad_input(lg, inst):
    with lg.Batch(4, 10000) as b:
        xy = inst.uniform_int(5000, 1)
        with pytest.raises(lg.LogoError):
            b.solve([xy], [np.arange(5000)], [1])
        xy = inst.uniform_int(50, 1)
        bad = np.arange(50)
        bad[3] = 4
        with pytest.raises(lg.LogoError):
            b.solve([xy], [bad], [1])
        with pytest.raises(lg.LogoError):
            b.solve([xy] * 5, [np.arange(50)] * 5, [1] * 5)


def test_multistart_independent_replicas_equal_ils(lg, inst):
    """Without sharing, replica k of a multi-start run is exactly logo_ils
    with seed + k, and the tour returned is the best replica's."""
    n, kicks, seed = 300, 30, 77
    xy = inst.uniform_f32(n, 3, 1.0e4)
    r = inst.random_tour(n, 4)
    with lg.Batch(8, 8 * n) as b:
        best_r, res, w, _ = b.multistart(xy, r, 6, seed, share=False, kicks=kicks)
    want = []
    with lg.Solver(xy) as s:
        for k in range(6):
            t, st = s.ils(r, kicks, seed + k, lg.KICK_SEGMENT)
            want.append((t, st))
    assert [x["best_length"] for x in res] == [st["final_length"] for _, st in want]
    assert [x["accepted"] for x in res] == [st["accepted"] for _, st in want]
    assert w == int(np.argmin([x["best_length"] for x in res]))
    assert np.array_equal(best_r, want[w][0])


def test_multistart_shared_single_replica_equals_ils(lg, inst):
    """A shared group of one replica publishes and adopts only its own best
    tour, which is what plain ILS reverts to."""
    n, kicks, seed = 500, 40, 5
    xy = inst.clustered(n, 6, side=1.0e6, clusters=5)
    r = inst.random_tour(n, 7)
    with lg.Batch(1, n) as b:
        got, res, w, _ = b.multistart(xy, r, 1, seed, share=True, kicks=kicks,
                                      kind=lg.KICK_DOUBLE_BRIDGE)
    with lg.Solver(xy) as s:
        want, st = s.ils(r, kicks, seed, lg.KICK_DOUBLE_BRIDGE)
    assert w == 0 and np.array_equal(got, want)
    assert res[0]["best_length"] == st["final_length"]
    assert res[0]["accepted"] == st["accepted"]


def test_multistart_shared_group(lg, inst, oracle_mod):
    """64 replicas sharing their best tour: every replica finishes, the tour
    returned is valid and as long as the best replica reports, and every
    replica's best is no worse than its start."""
    n, kicks, seed = 1000, 60, 11
    xy = inst.uniform_f32(n, 8, 1.0e4)
    r = inst.random_tour(n, 9)
    with lg.Batch(64, 64 * n) as b:
        got, res, w, ms = b.multistart(xy, r, 64, seed, share=True, kicks=kicks)
        again, res2, _, _ = b.multistart(xy, r, 64, seed, share=True, kicks=kicks)
    assert all(x["status"] == 0 and x["kicks"] == kicks for x in res + res2)
    assert lg.check_tour(got) and lg.check_tour(again)
    assert oracle_mod.tour_length(xy, got) == min(x["best_length"] for x in res)
    assert all(x["best_length"] <= x["start_length"] for x in res)
    assert ms > 0


@pytest.mark.parametrize("kicks", [0, 5])
def test_batch_nn_start_built_on_device(lg, inst, kicks):
    """start=START_NN: each CTA builds the nearest-neighbour tour of its
    instance; results equal the single-instance path started from the host
    logo_nn_tour (integer coordinates included: exact distance ties and
    duplicate points)."""
    coords, seeds = [], []
    for k, n in enumerate([50, 97, 300, 1000, 2000, 3000, 4096]):
        s = 700 + k
        if k % 3 == 0:
            xy = inst.uniform_int(n, s)
            xy = np.floor(xy / 50.0).astype(np.float32)  # many ties and duplicates
        elif k % 3 == 1:
            xy = inst.uniform_f32(n, s, 1.0e4)
        else:
            xy = inst.clustered(n, s, side=1.0e6, clusters=max(2, n // 200))
        coords.append(xy)
        seeds.append(s)
    total = sum(len(c) for c in coords)
    with lg.Batch(len(coords), total) as b:
        got, res, _ = b.solve(coords, None, seeds, kicks=kicks, start=lg.START_NN)
    for xy, g, r, s in zip(coords, got, res, seeds):
        nn = lg.nn_tour(xy, 0)
        with lg.Solver(xy) as sol:
            if kicks:
                want, st = sol.ils(nn, kicks, s, lg.KICK_SEGMENT)
                assert r["best_length"] == st["final_length"]
            else:
                want, st = sol.optimize(nn)
                assert r["best_length"] == st["final_length"]
            assert r["start_length"] == st["start_length"]
        assert np.array_equal(g, want), len(xy)


@pytest.mark.parametrize("kicks", [0, 4])
def test_batch_mf_start_built_on_device(lg, inst, kicks):
    """start=START_MF: a launch before the solve builds each instance's
    multiple-fragment tour (the host queue's order of equal distances
    replayed); start lengths and results equal the single-instance path
    started from the host logo_mf_tour.  Covered: 3-5 cities, integer grids
    with many equal distances and duplicate points, uniform and clustered
    instances up to the batch maximum of 4,096 cities."""
    coords, seeds = [], []
    for k, n in enumerate([3, 4, 5, 60, 97, 300, 1000, 2000, 3000, 4096]):
        s = 900 + k
        if k % 3 == 0:
            xy = inst.uniform_int(n, s)
            xy = np.floor(xy / 50.0).astype(np.float32)  # many ties and duplicates
        elif k % 3 == 1:
            xy = inst.uniform_f32(n, s, 1.0e4)
        else:
            xy = inst.clustered(n, s, side=1.0e6, clusters=max(2, n // 200))
        coords.append(xy)
        seeds.append(s)
    total = sum(len(c) for c in coords)
    with lg.Batch(len(coords), total) as b:
        got, res, _ = b.solve(coords, None, seeds, kicks=kicks, start=lg.START_MF)
    for xy, g, r, s in zip(coords, got, res, seeds):
        mf = lg.mf_tour(xy)
        assert r["status"] == 0
        with lg.Solver(xy) as sol:
            assert r["start_length"] == sol.route_length(mf), len(xy)
            if kicks:
                want, st = sol.ils(mf, kicks, s, lg.KICK_SEGMENT)
            else:
                want, st = sol.optimize(mf)
            assert r["best_length"] == st["final_length"]
        assert np.array_equal(g, want), len(xy)


def test_single_instance_start_tours_built_on_the_device(lg, inst):
    """logo_start_tour: a single-instance context's NN and MF start tours
    built by one CTA, equal to the host builders (ties and duplicate points
    included); above the one-CTA limit the call is refused."""
    for k, n in enumerate([3, 4, 5, 64, 1000, 2500, 4096]):
        for xy in (inst.uniform_f32(n, 60 + k, 1.0e4),
                   np.floor(inst.uniform_int(n, 70 + k) / 50.0).astype(np.float32)):
            with lg.Solver(xy) as s:
                assert np.array_equal(s.start_tour(lg.START_NN), lg.nn_tour(xy, 0)), n
                assert np.array_equal(s.start_tour(lg.START_MF), lg.mf_tour(xy)), n
    with lg.Solver(inst.uniform_f32(5000, 1, 1.0e4)) as s, pytest.raises(lg.LogoError):
        s.start_tour(lg.START_NN)
