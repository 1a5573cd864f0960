"""Index arithmetic of the boxed sweep, restated on the CPU (csrc/sweep.cu,
csrc/capi.cu make_tiles): the tile filter enumerates exactly the tiles of
the tile list (the work list holds one item per tile at most), every
window index it or the sweep forms stays inside the window-statistics
buffers, window boundaries line up with tile columns, and the filter's
grid covers every step of every row block."""
import pytest

WIN = 32


def make_tiles(n, rt, cb):
    # the host tile list: rows [row0, row0 + rt), columns [col0, col0 + cb)
    out = []
    if n < 4:
        return out
    row0 = 1
    while row0 + 3 <= n:
        col0 = row0 + 2
        while col0 <= n - 1:
            out.append((row0, col0))
            col0 += cb
        row0 += rt
    return out


def sweep_windows(n):
    return 1 if n < 4 else (n - 3 + 31) // 32


def filter_tiles(n, rt, cb):
    # tile_filter_kernel's enumeration and launch geometry
    row_blocks = (n - 4) // rt + 1
    wpt = cb // WIN
    tps = 32 // wpt
    steps = ((n - 3 + cb - 1) // cb + tps - 1) // tps
    grid_y = (steps + 7) // 8
    out = []
    for bx in range(row_blocks):
        row0 = 1 + bx * rt
        ntiles = (n - row0 - 2 + cb - 1) // cb
        covered = set()
        for by in range(grid_y):
            if by * 8 * tps >= ntiles:
                continue
            for warp in range(8):
                t0 = (by * 8 + warp) * tps
                while t0 < ntiles:
                    for lane in range(tps):
                        if t0 + lane < ntiles:
                            covered.add(t0 + lane)
                    t0 += grid_y * 8 * tps
        assert covered == set(range(ntiles)), (n, rt, cb, bx)
        out += [(row0, row0 + 2 + k * cb) for k in range(ntiles)]
    return out


SHAPES = [(4, 4, 64), (4, 4, 128), (4, 4, 256), (4, 4, 512), (4, 2, 96), (4, 8, 1024),
          (8, 4, 512), (8, 8, 1024), (16, 4, 1024), (4, 4, 32)]


@pytest.mark.parametrize("R,NW,cb", SHAPES)
def test_filter_enumerates_the_tile_list(R, NW, cb):
    rt = NW * 32 * R
    for n in (5, 6, 7, 34, 35, 36, 99, 100, 517, 1000, 4097, 17500, 33333, 100000):
        tiles = make_tiles(n, rt, cb)
        assert filter_tiles(n, rt, cb) == tiles, (n, R, NW, cb)


@pytest.mark.parametrize("R,NW,cb", SHAPES)
def test_window_indices_stay_in_bounds(R, NW, cb):
    rt = NW * 32 * R
    for n in (5, 7, 35, 36, 67, 68, 100, 1000, 4099, 100003):
        nwin = sweep_windows(n)
        for row0, col0 in make_tiles(n, rt, cb):
            assert (col0 - 3) % WIN == 0  # windows line up with tile columns
            col_end = min(col0 + cb, n)
            tile_windows = (col_end - col0 + WIN - 1) // WIN
            assert tile_windows <= 32  # one mask bit each
            last = (col0 - 3) // WIN + tile_windows - 1
            assert 0 <= last < nwin, (n, row0, col0)
            # the staged range [k0, k1) fits the tile's cb + 1 entries
            k1 = min(tile_windows * WIN, col_end - col0) + 1
            assert k1 <= cb + 1
            # row windows of the tile's rows with pairs
            row_end = min(row0 + rt, n - 2)
            assert (row0 - 1) % WIN == 0
            last_rw = (row0 - 1) // WIN + (row_end - row0 + WIN - 1) // WIN - 1
            assert last_rw < sweep_windows(n)
            assert (row_end - row0 + WIN - 1) // WIN <= 2048 // WIN
