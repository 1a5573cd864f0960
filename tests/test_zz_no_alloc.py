"""logo_best_move_noalloc against logo_best_move and the oracle, through the C ABI.

The allocation-free entry point serves callers that may not allocate device
memory themselves (pool-allocator owners, latency-sensitive loops that cannot
risk a device-synchronising cudaMalloc/cudaFree).  The test owns every buffer
(torch allocates them here, the entry point does not) and checks calls in a
row on different instances, so a later call must not see an earlier call's
leftovers in the shared static scratch array.  Results are integers and must
be identical.  Covered: the documented maximum n = 65,536 (the last word of
the permutation bitmap and the edge of the sweep grid), tours of 3 to 5
cities, a rejected call (non-finite coordinate) followed by a valid one, and
a coordinate pointer that is not 8-byte aligned.  This file is collected last
on purpose.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lg, torch, xy, route):
    n = len(route)
    d_xy = torch.from_numpy(np.ascontiguousarray(xy, dtype=np.float32)).cuda()
    d_route = torch.from_numpy(np.ascontiguousarray(route, dtype=np.uint32).view(np.int32)).cuda()
    d_out = torch.full((3,), -7, dtype=torch.int32, device="cuda")
    d_status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    lg.best_move_noalloc(d_xy.data_ptr(), d_route.data_ptr(), n, d_out.data_ptr(),
                         d_status.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    i, j, minchange = (int(v) for v in d_out.cpu().numpy().view(np.int32))
    i, j = i & 0xFFFFFFFF, j & 0xFFFFFFFF
    return (minchange, i, j), int(d_status.item())


def _oracle_move(oracle, xy, route):
    key = oracle.best_move_key(xy, route, threads=os.cpu_count() or 4)
    return (0, 0, 0) if key == (1 << 64) - 1 else oracle.unpack_key(key)


def test_noalloc_matches_best_move_on_two_calls(lg, inst):
    torch = pytest.importorskip("torch")
    cases = [(inst.uniform_f32(3001, 21, 1.0e6), inst.random_tour(3001, 21)),
             (inst.uniform_int(700, 22), inst.random_tour(700, 22))]
    for xy, route in cases:
        with lg.Solver(xy) as s:
            want = s.optimize_step(route)
        got, status = _noalloc(lg, torch, xy, route)
        assert status == 0
        assert got == want


def test_noalloc_at_its_maximum_and_small_tours(lg, inst, oracle_mod):
    torch = pytest.importorskip("torch")
    n = 65536  # LOGO_NOALLOC_MAX_CITIES
    xy = inst.uniform_f32(n, 23, 1.0e6)
    route = inst.random_tour(n, 23)
    got, status = _noalloc(lg, torch, xy, route)
    assert status == 0 and got == _oracle_move(oracle_mod, xy, route)
    with lg.Solver(xy) as s:
        assert s.optimize_step(route) == got
    square = np.array([[0, 0], [10, 0], [10, 10], [0, 10]], dtype=np.float32)
    small = [(square, np.array([0, 2, 1, 3], dtype=np.uint32))]
    for k, m in enumerate((3, 4, 5, 5, 4)):
        small.append((inst.uniform_int(m, 40 + k), inst.random_tour(m, 50 + k)))
    for xy, route in small:
        got, status = _noalloc(lg, torch, xy, route)
        assert status == 0 and got == oracle_mod.best_move(xy, route), (len(route), got)
    assert _noalloc(lg, torch, *small[0])[0] == (-8, 1, 3)


def test_noalloc_rejects_sizes_and_bad_routes(lg, inst):
    torch = pytest.importorskip("torch")
    # above LOGO_NOALLOC_MAX_CITIES: refused on the host before any device work
    with pytest.raises(lg.LogoError) as e:
        lg.best_move_noalloc(8, 8, 65537, 8)
    assert e.value.status == 1
    xy = inst.uniform_int(200, 3)
    bad = np.arange(200, dtype=np.uint32)
    bad[7] = 8
    got, status = _noalloc(lg, torch, xy, bad)
    assert status == 1 and got == (0, 0, 0)


def test_noalloc_after_a_rejected_call_and_misaligned_coordinates(lg, inst, oracle_mod):
    torch = pytest.importorskip("torch")
    n = 900
    xy = inst.uniform_f32(n, 31, 1.0e4)
    route = inst.random_tour(n, 31)
    nan_xy = xy.copy()
    nan_xy[17, 1] = np.nan
    got, status = _noalloc(lg, torch, nan_xy, route)
    assert status == 1 and got == (0, 0, 0)
    # the next call starts from cleared scratch
    got, status = _noalloc(lg, torch, xy, route)
    assert status == 0 and got == oracle_mod.best_move(xy, route)
    # coordinates at an odd float offset (4-byte, not 8-byte aligned): refused
    flat = torch.zeros(2 * n + 1, dtype=torch.float32, device="cuda")
    flat[1:] = torch.from_numpy(xy.reshape(-1)).cuda()
    d_route = torch.from_numpy(route.view(np.int32)).cuda()
    d_out = torch.zeros(3, dtype=torch.int32, device="cuda")
    with pytest.raises(lg.LogoError) as e:
        lg.best_move_noalloc(flat.data_ptr() + 4, d_route.data_ptr(), n, d_out.data_ptr(),
                             None, torch.cuda.current_stream().cuda_stream)
    assert e.value.status == 1
    # and the entry point still answers correctly afterwards
    got, status = _noalloc(lg, torch, xy, route)
    assert status == 0 and got == oracle_mod.best_move(xy, route)
