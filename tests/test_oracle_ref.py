"""The oracle against the reference's own compiled code, live (CPU only).

Needs oracle/_ref/ref_harness (oracle/build_ref.sh: the reference checkout on
an x86-64 host); skipped elsewhere.  The golden fixtures carry the same
checks to hosts without the reference.
"""
import numpy as np
import pytest

ref = pytest.importorskip("ref")
pytestmark = pytest.mark.skipif(not ref.available(), reason="reference harness not built")


@pytest.mark.parametrize("seed", range(6))
def test_step_and_descent(oracle_mod, inst, seed):
    n = [7, 40, 150, 300, 401, 250][seed]
    xy = inst.uniform_f32(n, seed, 1.0e3) if seed % 2 else inst.uniform_int(n, seed)
    r = inst.random_tour(n, seed + 50)
    assert oracle_mod.best_move(xy, r) == ref.step(xy, r)
    fr, m, log, length = ref.descend(xy, r)
    fo, mo, logo = oracle_mod.descend(xy, r, log_cap=1 << 20)
    assert (m, length) == (mo, oracle_mod.tour_length(xy, fo))
    assert np.array_equal(log, logo) and np.array_equal(fr, fo)
    assert ref.length(xy, r) == oracle_mod.tour_length(xy, r)


def test_tours_of_four_to_six_cities(oracle_mod, inst):
    """The reference's loop bounds (i < n-2, j < n-1) leave one pair at n = 4."""
    for seed in range(12):
        for n in (4, 5, 6):
            xy = inst.uniform_int(n, seed)
            r = inst.random_tour(n, seed + 7)
            assert oracle_mod.best_move(xy, r) == ref.step(xy, r), (n, seed)
            fr, m, log, length = ref.descend(xy, r)
            fo, mo, logo = oracle_mod.descend(xy, r, log_cap=64)
            assert m == mo and np.array_equal(fr, fo) and np.array_equal(log, logo)


def test_duplicate_points_and_ties(oracle_mod, inst):
    rng = np.random.default_rng(1)
    xy = np.floor(rng.random((120, 2)) * 8).astype(np.float32)
    r = inst.random_tour(120, 9)
    fr, m, log, length = ref.descend(xy, r)
    fo, mo, logo = oracle_mod.descend(xy, r, log_cap=1 << 20)
    assert np.array_equal(log, logo) and np.array_equal(fr, fo)


def test_kick_and_ils(oracle_mod, inst):
    xy = inst.uniform_f32(120, 4, 1.0e4)
    r = inst.random_tour(120, 4)
    rk, st = ref.kick(xy, r, 99, 7)
    ok, s = r, 99
    for _ in range(7):
        ok, s = oracle_mod.kick(ok, s)
    assert np.array_equal(rk, ok) and st == s
    br, bl, moves = ref.ils(xy, r, 15, 3)
    bo, ost = oracle_mod.ils(xy, r, 15, 3)
    assert np.array_equal(br, bo) and bl == ost["best_length"] and moves == ost["moves"]


def test_avx_reference_is_close(oracle_mod, inst):
    """The shipped AVX CPUSolver uses x*rsqrt(x) (relative error up to
    1.5*2^-12 for rsqrtps) and no per-edge rounding (src/utils/cpusimd.h,
    src/solvers/cpuSolver.cpp:151-197), so its first move's delta is only
    within 2 + 4 * 1.5*2^-12 * diagonal of the per-edge nint delta."""
    diag = (2 * 1.0e4 ** 2) ** 0.5
    tol = 2 + 4 * 1.5 * 2.0 ** -12 * diag
    same = 0
    for seed in range(8):
        xy = inst.uniform_int(500, seed)
        r = inst.random_tour(500, seed)
        d_avx, i_avx, j_avx = ref.avx_step(xy, r)
        d, i, j = oracle_mod.best_move(xy, r)
        assert abs(d_avx - d) <= tol
        same += (i_avx, j_avx) == (i, j)
    assert same >= 6


def test_nn_tour(oracle_mod, inst):
    xy = inst.clustered(3000, 4)
    t, ties = oracle_mod.nn_tour(xy)
    assert ties == 0
    assert np.array_equal(ref.nn_tour(xy), t)


def test_mf_tour_live(lg, inst):
    """The library's multiple-fragment tour against the reference's, run now,
    on fresh seeds (the fixtures hold other seeds)."""
    for n, seed in ((777, 31), (4000, 32), (15000, 33)):
        xy = inst.clustered(n, seed, side=1.0e6, clusters=max(2, n // 100))
        assert np.array_equal(lg.mf_tour(xy), ref.mf_tour(xy)), n
