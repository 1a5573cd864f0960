"""The drop-in boundary, compiled for real.

* integration/GPUSolver.h, the TwoOptLocalSolver subclass a maintainer adds to
  the reference tree, compiled against the reference's own headers
  (src/solvers/localSolver.h:25-132, twoOptLocalSolver.h:23-70, src/defs.h)
  and linked with the reference's twoOptLocalSolver.cpp and common.c and with
  liblogo_gpu.so.  Needs the reference checkout (REF, default
  /root/reference); skipped without it.
* tests/c/abi_smoke.c, a plain C program that calls create, best move,
  descend, tour length, ILS, the device start tours, the neighbour-list
  search, the copied route transfer and destroy through include/logo_gpu.h:
  compiled here with -Wall -Werror, and run on a GPU against the oracle and
  the host builders.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("REF", "/root/reference")
INCLUDE = os.path.join(ROOT, "include")


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    assert r.returncode == 0, (cmd, r.stdout, r.stderr)
    return r


def _link_flags(lg):
    libdir = os.path.dirname(os.path.abspath(lg.LIB_PATH))
    return [f"-L{libdir}", "-llogo_gpu", f"-Wl,-rpath,{libdir}"]


def test_gpu_solver_adapter_compiles_and_links_against_the_reference(lg, tmp_path):
    if not os.path.isdir(os.path.join(REF, "src", "solvers")):
        pytest.skip("no reference checkout")
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    inc = [f"-I{REF}/src", f"-I{REF}/src/solvers", f"-I{REF}/src/utils", f"-I{INCLUDE}",
           f"-I{os.path.join(ROOT, 'integration')}"]
    objs = []
    for src, lang in ((os.path.join(ROOT, "tests", "c", "gpu_solver_link.cpp"), "c++"),
                      (f"{REF}/src/solvers/twoOptLocalSolver.cpp", "c++"),
                      (f"{REF}/src/utils/common.c", "c++")):
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        _run(["g++", "-x", lang, "-std=c++11", "-O1", "-Wall", *inc, "-c", src, "-o", obj])
        objs.append(obj)
    exe = str(tmp_path / "gpu_solver_link")
    _run(["g++", *objs, *_link_flags(lg), "-o", exe])
    _run([exe])  # no arguments: every symbol resolved, no device touched


def _build_smoke(lg, tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    exe = str(tmp_path / "abi_smoke")
    _run(["gcc", "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{INCLUDE}",
          os.path.join(ROOT, "tests", "c", "abi_smoke.c"), *_link_flags(lg), "-o", exe])
    return exe


def test_c_abi_smoke_compiles(lg, tmp_path):
    _build_smoke(lg, tmp_path)


@pytest.mark.gpu
def test_c_abi_smoke_program_matches_the_oracle(lg, inst, oracle_mod, tmp_path):
    exe = _build_smoke(lg, tmp_path)
    n = 700
    xy = inst.uniform_f32(n, 13, 1.0e4)
    r = inst.random_tour(n, 14)
    path = tmp_path / "instance.bin"
    with open(path, "wb") as f:
        f.write(struct.pack("<I", n))
        f.write(np.ascontiguousarray(xy, dtype=np.float32).tobytes())
        f.write(np.ascontiguousarray(r, dtype=np.uint32).tobytes())
    out = _run([exe, str(path)], timeout=300).stdout.splitlines()
    rows = {ln.split()[0]: [int(v) for v in ln.split()[1:]] for ln in out}
    assert tuple(rows["move"]) == oracle_mod.best_move(xy, r)
    want, m, _ = oracle_mod.descend(xy, r)
    assert rows["descend"][0] == m
    assert rows["descend"][1] == oracle_mod.tour_length(xy, want)
    assert np.array_equal(np.array(rows["descend"][2:], dtype=np.uint32), want)
    assert rows["length"][0] == oracle_mod.tour_length(xy, want)
    best, st = oracle_mod.ils(xy, r, 10, 99, oracle_mod.KICK_DOUBLE_BRIDGE)
    assert rows["ils"][:3] == [st["best_length"], st["moves"], st["accepted"]]
    assert np.array_equal(np.array(rows["ils"][3:], dtype=np.uint32), best)
    assert np.array_equal(np.array(rows["nnstart"], dtype=np.uint32), lg.nn_tour(xy, 0))
    assert np.array_equal(np.array(rows["mfstart"], dtype=np.uint32), lg.mf_tour(xy))
    nb, nm, _ = oracle_mod.descend_nbr(xy, r, k=8)
    assert rows["nbrdescend"][0] == nm
    assert np.array_equal(np.array(rows["nbrdescend"][2:], dtype=np.uint32), nb)
    assert rows["copydescend"] == [m, oracle_mod.tour_length(xy, want)]
