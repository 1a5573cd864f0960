"""The C-ABI library loads and exports every function include/logo_gpu.h
declares.  CPU only: no call here launches GPU work."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(logo_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("logo_ctx_create", "logo_best_move", "logo_descend", "logo_ils",
                 "logo_tour_length", "logo_ctx_destroy", "logo_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lg):
    lib = ctypes.CDLL(lg.LIB_PATH)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(lg.EXPORTS) <= declared_functions()


def test_exports_are_dynamic_symbols(lg):
    out = subprocess.run(["nm", "-D", "--defined-only", lg.LIB_PATH], capture_output=True,
                         text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if " T " in ln}
    assert declared_functions() <= exported


def test_version_and_error_path_without_compute(lg):
    L = lg.load()
    assert b"sm_103a" in L.logo_version()
    # invalid arguments are rejected on the host before any device work
    h = ctypes.c_void_p()
    assert L.logo_ctx_create(0, None, 10, ctypes.byref(h)) == 1
    assert b"NULL" in L.logo_last_error(None)
    assert L.logo_best_move(None, None, None) == 1
    assert L.logo_ctx_destroy(None) == 0
    assert L.logo_ctx_set_kernel(None, lg.SWEEP_BOXED, 4, 4, 128) == 1
    assert L.logo_ctx_set_descent_mode(None, lg.DESCENT_GRAPH) == 1
    assert L.logo_diag_wait_limits(0, None, None, None) == 1
