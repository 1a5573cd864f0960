"""Request server: continuous batching must not change any result.

Each request's tour, length and move count must be identical when it runs
alone, when it runs mixed with others (arriving while they are on the GPU), and
when it runs through the single-instance path (logo_ils) -- the tolerance is
zero: all quantities are integers."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(inst, count, seed, large=()):
    out = []
    ns = list(inst.batch_sizes(count, seed, 40, 2500)) + list(large)
    for k, n in enumerate(ns):
        s = inst.instance_seed(seed, k)
        xy = inst.uniform_f32(int(n), s, 1.0e4) if k % 2 else inst.clustered(int(n), s)
        out.append((xy, inst.random_tour(int(n), s), s))
    return out


def test_results_same_alone_in_mix_and_single_instance(lg, inst):
    reqs = _requests(inst, 18, 4, large=(4500, 5200))
    kicks = 4
    alone = []
    with lg.Server(kicks=kicks) as srv:
        for xy, r, s in reqs:
            rid = srv.submit(xy, r, s)
            alone.append(srv.wait(rid))
    with lg.Server(kicks=kicks, quantum_pairs=2_000_000) as srv:
        ids = [srv.submit(xy, r, s) for xy, r, s in reqs]
        mixed = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["rounds"] > 1
    for (ra, ia), (rm, im), (xy, r, s) in zip(alone, mixed, reqs):
        assert ia["status"] == 0 and im["status"] == 0
        assert np.array_equal(ra, rm)
        assert ia["best_length"] == im["best_length"]
        assert ia["moves"] == im["moves"] and ia["accepted"] == im["accepted"]
    for (rm, im), (xy, r, s) in list(zip(mixed, reqs))[::4]:
        with lg.Solver(xy) as sol:
            want, stt = sol.ils(r, kicks, s, lg.KICK_SEGMENT)
        assert np.array_equal(rm, want)
        assert im["best_length"] == stt["final_length"]


def test_admission_respects_memory_budget(lg, inst):
    reqs = _requests(inst, 10, 7)
    biggest = max(len(r) for _, r, _ in reqs)
    budget = 16 * biggest * 2  # room for about two resident requests
    with lg.Server(kicks=2, mem_budget=budget) as srv:
        ids = [srv.submit(xy, r, s) for xy, r, s in reqs]
        peak = 0
        while True:
            st = srv.stats()
            peak = max(peak, st["mem_in_use"])
            if st["completed"] == len(reqs):
                break
            time.sleep(0.002)
        res = [srv.wait(i) for i in ids]
    assert peak <= budget
    assert all(info["status"] == 0 for _, info in res)
    # later requests had to wait for memory
    assert max(info["queue_ms"] for _, info in res) > 0


def test_requests_join_while_others_run(lg, inst):
    long_xy = inst.uniform_f32(3500, 1, 1.0e4)
    long_r = inst.random_tour(3500, 1)
    short = _requests(inst, 6, 9)
    with lg.Server(kicks=20, quantum_pairs=1_000_000) as srv:
        big = srv.submit(long_xy, long_r, 5)
        time.sleep(0.05)
        ids = [srv.submit(xy, r, s) for xy, r, s in short]
        res = [srv.wait(i) for i in ids]
        assert srv.poll(big) is None or True  # may or may not be done yet
        rbig, ibig = srv.wait(big)
    # the short requests finished while the long one was still in flight
    assert max(info["latency_ms"] for _, info in res) < ibig["latency_ms"]
    with lg.Solver(long_xy) as sol:
        want, st = sol.ils(long_r, 20, 5, lg.KICK_SEGMENT)
    assert np.array_equal(rbig, want)


def test_server_errors(lg, inst):
    with lg.Server(kicks=0) as srv:
        xy = inst.uniform_int(30, 1)
        bad = np.arange(30)
        bad[1] = 0
        with pytest.raises(lg.LogoError):
            srv.submit(xy, bad, 1)
        rid = srv.submit(xy, np.arange(30), 1)
        srv.wait(rid)
        with pytest.raises(KeyError):
            srv.poll(rid)  # consumed
