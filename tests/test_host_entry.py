"""Host-side entry points of the library (instance parse, start tours, tour
check) against the reference's own outputs.  CPU only."""
import hashlib
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the reference checkout (the same REF variable oracle/build_ref.sh reads)
REF_TSPLIB = os.path.join(os.environ.get("REF", "/root/reference"), "TSPLIB")
GENS = ["uniform_int", "uniform_f32", "clustered"]


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_nn_tour_matches_reference_kdtree(lg, inst):
    g = np.load(os.path.join(GOLD, "nn_tours.npz"))
    for (gi, n, seed), h, out in zip(g["spec"], g["hash"], g["out"]):
        n, seed = int(n), int(seed)
        if GENS[gi] == "uniform_int":
            xy = inst.uniform_int(n, seed)
        elif GENS[gi] == "uniform_f32":
            xy = inst.uniform_f32(n, seed, 1.0e4)
        else:
            xy = inst.clustered(n, seed, side=1.0e6, clusters=max(2, n // 50))
        assert digest(xy) == h
        assert digest(lg.nn_tour(xy, 0)) == out


@pytest.mark.parametrize("name", ["berlin52", "kroA100", "pr2392"])
def test_nn_tour_tsplib(lg, oracle_mod, name):
    """Identical to the reference kd-tree tour where no two candidates are
    equidistant (berlin52, kroA100).  pr2392 has exact distance ties, which
    the kd-tree breaks by traversal order and this library by lowest id: the
    tours must then agree up to the first tie, and that step must be a tie."""
    g = np.load(os.path.join(GOLD, "tsplib.npz"))
    xy, want = g[name + "_xy"], g[name + "_nn"]
    got = lg.nn_tour(xy, 0)
    t, ties = oracle_mod.nn_tour(xy)
    assert np.array_equal(got, t)
    if ties == 0:
        assert np.array_equal(got, want)
    else:
        k = int(np.nonzero(got != want)[0][0])
        prev = xy[want[k - 1]].astype(np.float64)
        d = [np.sqrt(((xy[c].astype(np.float64) - prev) ** 2).sum()) for c in (got[k], want[k])]
        assert d[0] == d[1] and got[k] < want[k]


def _instance(inst, gi, n, seed):
    if GENS[gi] == "uniform_int":
        return inst.uniform_int(n, seed)
    if GENS[gi] == "uniform_f32":
        return inst.uniform_f32(n, seed, 1.0e4)
    return inst.clustered(n, seed, side=1.0e6, clusters=max(2, n // 50))


def test_mf_tour_matches_reference(lg, inst):
    """Multiple-fragment tours equal the reference's multipleFragment_KD on
    every fixture (n = 3..10,000; float, clustered and integer coordinates)."""
    g = np.load(os.path.join(GOLD, "mf_tours.npz"))
    for (gi, n, seed), h, out in zip(g["spec"], g["hash"], g["out"]):
        xy = _instance(inst, gi, int(n), int(seed))
        assert digest(xy) == h
        assert digest(lg.mf_tour(xy)) == out, (GENS[gi], int(n), int(seed))


@pytest.mark.parametrize("name", ["berlin52", "kroA100", "att532"])
def test_mf_tour_tsplib(lg, name):
    g = np.load(os.path.join(GOLD, "mf_tours.npz"))
    assert np.array_equal(lg.mf_tour(g[name + "_xy"]), g[name + "_mf"])


def test_mf_tour_edge_cases(lg, inst):
    assert list(lg.mf_tour(np.zeros((1, 2), np.float32))) == [0]
    assert list(lg.mf_tour(np.array([[0, 0], [3, 4]], np.float32))) == [0, 1]
    dup = np.array([[0, 0], [5, 5], [0, 0], [1, 0], [5, 5], [9, 1]], dtype=np.float32)
    assert lg.check_tour(lg.mf_tour(dup))
    xy = inst.clustered(30000, 4, side=1.0e6, clusters=60)
    assert lg.check_tour(lg.mf_tour(xy))
    bad = inst.uniform_f32(10, 1, 1.0e4)
    bad[3, 1] = np.nan
    with pytest.raises(lg.LogoError):
        lg.mf_tour(bad)


def test_nn_tour_keeps_duplicates(lg):
    xy = np.array([[0, 0], [5, 5], [0, 0], [1, 0], [5, 5]], dtype=np.float32)
    t = lg.nn_tour(xy, 0)
    assert lg.check_tour(t) and t[0] == 0 and t[1] == 2


def test_random_tour_matches_generator(lg, inst):
    for n, seed in ((5, 1), (1000, 7), (65537, 3)):
        t = lg.random_tour(n, seed)
        assert np.array_equal(t, inst.random_tour(n, seed))
        assert lg.check_tour(t)


def test_check_tour(lg):
    assert lg.check_tour(np.array([2, 0, 1]))
    assert not lg.check_tour(np.array([0, 1, 1]))
    assert not lg.check_tour(np.array([0, 1, 3]))
    assert not lg.check_tour(np.array([1, 0]))


def test_read_tsplib_written_file(lg, tmp_path):
    xy = np.array([[1.5, 2.25], [1e6, 3.0], [-4.0, 7.5], [0.0, 0.0]], dtype=np.float32)
    p = tmp_path / "t.tsp"
    lines = ["NAME : t", "COMMENT : a comment", "COMMENT : a second comment line",
             "TYPE : TSP", "DIMENSION : 4", "EDGE_WEIGHT_TYPE : EUC_2D", "NODE_COORD_SECTION"]
    lines += [f"{k + 1} {x:.6e} {y:.6e}" for k, (x, y) in enumerate(xy)] + ["EOF"]
    p.write_text("\n".join(lines) + "\n")
    assert np.array_equal(lg.read_tsplib(str(p)), xy)


def test_read_tsplib_rejects_bad_files(lg, tmp_path):
    p = tmp_path / "bad.tsp"
    p.write_text("<html><body>not a tsp</body></html>\n")
    with pytest.raises(lg.LogoError):
        lg.read_tsplib(str(p))
    p.write_text("DIMENSION : 5\nNODE_COORD_SECTION\n1 0 0\n2 1 1\nEOF\n")
    with pytest.raises(lg.LogoError):
        lg.read_tsplib(str(p))
    with pytest.raises(lg.LogoError) as e:
        lg.read_tsplib(str(tmp_path / "missing.tsp"))
    assert e.value.status == 9


@pytest.mark.skipif(not os.path.isdir(REF_TSPLIB), reason="reference checkout not present")
@pytest.mark.parametrize("name", ["berlin52", "kroA100", "pr2392", "a280", "usa13509"])
def test_read_tsplib_matches_reference_reader(lg, name):
    ref = pytest.importorskip("ref")
    if not ref.available():
        pytest.skip("reference harness not built")
    path = os.path.join(REF_TSPLIB, name + ".tsp")
    assert np.array_equal(lg.read_tsplib(path), ref.read_tsp(path))


def test_read_tsplib_fixture_coordinates(lg, tmp_path):
    """Round trip of the reference-parsed berlin52 coordinates."""
    g = np.load(os.path.join(GOLD, "tsplib.npz"))
    xy = g["berlin52_xy"]
    p = tmp_path / "b.tsp"
    p.write_text("NAME: b\nTYPE: TSP\nDIMENSION: %d\nNODE_COORD_SECTION\n" % len(xy) +
                 "".join(f"{k + 1} {float(x)!r} {float(y)!r}\n" for k, (x, y) in
                         enumerate(xy.astype(np.float64))) + "EOF\n")
    assert np.array_equal(lg.read_tsplib(str(p)), xy)


def test_tour_files_round_trip(lg, inst, tmp_path):
    r = inst.random_tour(777, 5)
    for header in (True, False):
        p = str(tmp_path / f"t{int(header)}.tour")
        lg.write_tour(p, r, name="t777", tsplib_header=header)
        assert np.array_equal(lg.read_tour(p), r)
    text = open(str(tmp_path / "t1.tour")).read()
    assert text.startswith("NAME : t777\n") and "TOUR_SECTION\n" in text
    assert text.endswith("-1\nEOF\n")
    assert open(str(tmp_path / "t0.tour")).read().split()[:3] == [str(v + 1) for v in r[:3]]


def test_read_tour_formats_and_errors(lg, tmp_path):
    p = tmp_path / "a.tour"
    p.write_text("NAME : a\nCOMMENT : x\nTYPE : TOUR\nDIMENSION : 5\nTOUR_SECTION\n"
                 "3 1\n5\n 2 4 -1\nEOF\n")
    assert list(lg.read_tour(str(p))) == [2, 0, 4, 1, 3]
    p.write_text("2\n1\n3\n")  # the reference's bare list
    assert list(lg.read_tour(str(p))) == [1, 0, 2]
    for bad in ("DIMENSION : 4\nTOUR_SECTION\n1 2 3\n-1\n",  # too short
                "TOUR_SECTION\n1 2 2\n-1\n",                  # repeated id
                "TOUR_SECTION\n1 0 2\n-1\n",                  # 0 is not an id
                "TOUR_SECTION\n1 4 2\n-1\n",                  # gap in the ids
                "TOUR_SECTION\n-1\n"):
        p.write_text(bad)
        with pytest.raises(lg.LogoError):
            lg.read_tour(str(p))
    with pytest.raises(lg.LogoError):
        lg.read_tour(str(tmp_path / "missing.tour"))
    with pytest.raises(lg.LogoError):
        lg.write_tour(str(tmp_path / "w.tour"), np.array([0, 0, 1]))


def test_tsplib_info(lg, tmp_path):
    p = tmp_path / "c.tsp"
    p.write_text("NAME : c\nTYPE : TSP\nDIMENSION : 3\nEDGE_WEIGHT_TYPE : CEIL_2D\n"
                 "NODE_COORD_SECTION\n1 0 0\n2 3 4\n3 6 8\nEOF\n")
    assert lg.tsplib_info(str(p)) == (3, "CEIL_2D")
    p.write_text("NAME : d\nDIMENSION: 3\nNODE_COORD_SECTION\n1 0 0\n2 3 4\n3 6 8\n")
    assert lg.tsplib_info(str(p)) == (3, "EUC_2D")


@pytest.mark.skipif(not os.path.isdir(REF_TSPLIB), reason="reference TSPLIB files absent")
@pytest.mark.parametrize("name,ewt", [("berlin52", "EUC_2D"), ("att532", "ATT"),
                                      ("pla7397", "CEIL_2D")])
def test_tsplib_info_reference_files(lg, name, ewt):
    n, t = lg.tsplib_info(os.path.join(REF_TSPLIB, name + ".tsp"))
    assert t == ewt and n == int(name.lstrip("abcdefghijklmnopqrstuvwxyz"))
