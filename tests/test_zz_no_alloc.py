"""logo_best_move_noalloc against logo_best_move, through the C ABI.

The allocation-free entry point serves callers that may not allocate device
memory themselves (pool-allocator owners, latency-sensitive loops that cannot
risk a device-synchronising cudaMalloc/cudaFree).  The test owns every buffer
(torch allocates them here, the entry point does not) and checks two calls in
a row on different instances, so a second call must not see the first call's
leftovers in the shared static scratch array.  Results are integers and must
be identical.  This file is collected last on purpose.
"""
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


def test_noalloc_rejects_sizes_and_bad_routes(lg, inst):
    torch = pytest.importorskip("torch")
    # above LOGO_NOALLOC_MAX_CITIES: refused on the host before any device work
    with pytest.raises(lg.LogoError) as e:
        lg.best_move_noalloc(1, 1, 65537, 1)
    assert e.value.status == 1
    xy = inst.uniform_int(200, 3)
    bad = np.arange(200, dtype=np.uint32)
    bad[7] = 8
    got, status = _noalloc(lg, torch, xy, bad)
    assert status == 1 and got == (0, 0, 0)
