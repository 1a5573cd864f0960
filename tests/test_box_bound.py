"""The boxed screen's window test never closes a block that holds a pair the
sweep could choose (CPU check of the bound in sweep_core7.cuh).

A pair (i, c) can only be chosen when its reference distance
d1 = (int)(sqrtf(dx*dx + dy*dy) + 0.5f) is at most V = B + e[i] + e[c]
(e = incoming edge lengths, B <= -1 the best delta known).  The kernels
skip a block of rows and a 32-column window when
    s = RN(gy^2 + RN(gx^2)) >= RN(u^2),  u = B + max e[i] + 5 + max e[c],
gx, gy the binary32 gaps between the two bounding boxes.  Here every block
of seeded instances is checked in binary32 emulation: whenever some pair
of the block could be chosen, the test must keep the block open.
"""
import numpy as np
import pytest

F = np.float32


def _nint(ax, ay, bx, by):
    # the reference's distance: binary32, no contraction, sqrt rounded once
    dx = (ax - bx).astype(F)
    dy = (ay - by).astype(F)
    s = ((dx * dx).astype(F) + (dy * dy).astype(F)).astype(F)
    return (np.sqrt(s).astype(F) + F(0.5)).astype(F).astype(np.int64)


def _fma32(a, b, c):
    # RN(a*b + c) for binary32 inputs: the product is exact in binary64
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


def _box_pass(rbox, wbox, u):
    """The kernels' test (box_gap_pass) on arrays of boxes (x0, x1, y0, y1)."""
    gx = np.maximum(np.maximum((wbox[..., 0] - rbox[..., 1]).astype(F),
                               (rbox[..., 0] - wbox[..., 1]).astype(F)), F(0))
    gy = np.maximum(np.maximum((wbox[..., 2] - rbox[..., 3]).astype(F),
                               (rbox[..., 2] - wbox[..., 3]).astype(F)), F(0))
    s = _fma32(gy, gy, (gx * gx).astype(F))
    u = u.astype(F)
    return (u > 0) & (s < (u * u).astype(F))


def _instances(inst):
    out = []
    xy = inst.clustered(3000, 5, side=1.0e6, clusters=12, sigma_frac=0.01)
    out.append(("clustered_random", xy, inst.random_tour(3000, 6)))
    out.append(("clustered_sorted", xy, np.lexsort((xy[:, 1], xy[:, 0])).astype(np.uint32)))
    xy = inst.uniform_f32(2500, 7, 1.0e6)
    out.append(("uniform_sorted", xy, np.argsort(xy[:, 0]).astype(np.uint32)))
    xy = inst.uniform_int(2500, 8)
    out.append(("integer_random", xy, inst.random_tour(2500, 9)))
    # a diagonal-sized box, coordinates near the library's limit
    rng = np.random.default_rng(10)
    xy = rng.uniform(0, 1.4e6, size=(1500, 2)).astype(F)
    out.append(("large_box_sorted", xy, np.argsort(xy[:, 1]).astype(np.uint32)))
    return out


@pytest.mark.parametrize("B", [-1, -7, -500])
@pytest.mark.parametrize("rows", [1, 4])
def test_box_test_keeps_every_choosable_block(inst, B, rows):
    checked = closed = 0
    for name, xy, route in _instances(inst):
        q = xy[route].astype(F)
        n = len(q)
        x, y = q[:, 0], q[:, 1]
        e = np.empty(n, np.int64)
        e[1:] = _nint(x[1:], y[1:], x[:-1], y[:-1])
        e[0] = _nint(x[:1], y[:1], x[-1:], y[-1:])[0]
        ncw = (n - 3) // 32
        cols = 3 + np.arange(ncw * 32).reshape(ncw, 32)
        wbox = np.stack([x[cols].min(1), x[cols].max(1), y[cols].min(1), y[cols].max(1)], -1)
        wmax = e[cols].max(1)
        for i0 in range(1, n - 3, rows):
            ri = np.arange(i0, min(i0 + rows, n - 2))
            rbox = np.array([x[ri].min(), x[ri].max(), y[ri].min(), y[ri].max()], F)
            u = (B + e[ri].max() + 5 + wmax).astype(np.float64)
            keep = _box_pass(rbox[None, :], wbox, u)
            # which windows hold a choosable pair (c >= i + 2)
            d1 = _nint(x[ri][:, None, None], y[ri][:, None, None], x[cols][None], y[cols][None])
            V = B + e[ri][:, None, None] + e[cols][None]
            ok = (d1 <= V) & (cols[None] >= ri[:, None, None] + 2)
            need = ok.any(axis=(0, 2))
            assert not (need & ~keep).any(), (name, B, rows, i0, np.nonzero(need & ~keep))
            checked += int(need.sum())
            closed += int((~keep).sum())
    assert checked > 0 and closed > 0  # the test was exercised both ways


@pytest.mark.parametrize("bsel", ["minus_one", "true_best", "true_best_plus_7"])
def test_tile_filter_bound_keeps_every_choosable_block(inst, oracle_mod, bsel):
    """The filter's form: 32-row windows against 32-column windows with
    u = B + 5 + E_r + E_c (largest incoming edges of the two windows), B = -1
    or the seed pass's bound.  A seed is a real pair's delta, so it is never
    below the sweep's best delta; the tightest B a seed can give is that best
    delta itself, checked here together with a looser one.  Also the filter's
    block test (the union of a row block's windows) in front of the
    per-window tests: it must pass wherever one of its windows passes."""
    checked = 0
    for name, xy, route in _instances(inst):
        B = -1
        if bsel != "minus_one":
            d, _, _ = oracle_mod.best_move(xy, route)
            if d == 0:
                continue
            B = min(-1, d + (7 if bsel == "true_best_plus_7" else 0))
        q = xy[route].astype(F)
        n = len(q)
        x, y = q[:, 0], q[:, 1]
        e = np.empty(n, np.int64)
        e[1:] = _nint(x[1:], y[1:], x[:-1], y[:-1])
        e[0] = _nint(x[:1], y[:1], x[-1:], y[-1:])[0]
        ncw = (n - 3) // 32
        cols = 3 + np.arange(ncw * 32).reshape(ncw, 32)
        wbox = np.stack([x[cols].min(1), x[cols].max(1), y[cols].min(1), y[cols].max(1)], -1)
        wmax = e[cols].max(1)
        nrw = (n - 3) // 32
        rws = 1 + np.arange(nrw * 32).reshape(nrw, 32)
        rbox = np.stack([x[rws].min(1), x[rws].max(1), y[rws].min(1), y[rws].max(1)], -1)
        rmax = e[rws].max(1)
        u = ((rmax[:, None] + F(B + 5)).astype(F) + wmax[None, :]).astype(np.float64)
        keep = _box_pass(rbox[:, None, :], wbox[None, :, :], u)
        # row blocks of 16 windows (512 rows): union box and largest edge
        for b0 in range(0, nrw, 16):
            blk = slice(b0, min(b0 + 16, nrw))
            ubox = np.array([rbox[blk, 0].min(), rbox[blk, 1].max(), rbox[blk, 2].min(),
                             rbox[blk, 3].max()], F)
            uu = ((F(rmax[blk].max()) + F(B + 5)).astype(F) + wmax).astype(np.float64)
            ukeep = _box_pass(ubox[None, :], wbox, uu)
            assert not (keep[blk].any(axis=0) & ~ukeep).any(), (name, b0)
        for r in range(nrw):
            ri = rws[r]
            d1 = _nint(x[ri][:, None, None], y[ri][:, None, None], x[cols][None], y[cols][None])
            V = B + e[ri][:, None, None] + e[cols][None]
            ok = (d1 <= V) & (cols[None] >= ri[:, None, None] + 2)
            need = ok.any(axis=(0, 2))
            assert not (need & ~keep[r]).any(), (name, r, np.nonzero(need & ~keep[r]))
            checked += int(need.sum())
    assert checked > 0


@pytest.mark.parametrize("rows", [1, 4])
def test_box_test_at_the_critical_best_delta(inst, rows):
    """The sharpest case: for every block, B set to the largest value at which
    the block still holds a choosable pair (B = min over its pairs of
    d1 - e[i] - e[c], when that is <= -1), so that only its critical pairs
    keep it open."""
    tested = 0
    for name, xy, route in _instances(inst):
        q = xy[route].astype(F)
        n = len(q)
        x, y = q[:, 0], q[:, 1]
        e = np.empty(n, np.int64)
        e[1:] = _nint(x[1:], y[1:], x[:-1], y[:-1])
        e[0] = _nint(x[:1], y[:1], x[-1:], y[-1:])[0]
        ncw = (n - 3) // 32
        cols = 3 + np.arange(ncw * 32).reshape(ncw, 32)
        wbox = np.stack([x[cols].min(1), x[cols].max(1), y[cols].min(1), y[cols].max(1)], -1)
        wmax = e[cols].max(1)
        for i0 in range(1, n - 3, rows):
            ri = np.arange(i0, min(i0 + rows, n - 2))
            d1 = _nint(x[ri][:, None, None], y[ri][:, None, None], x[cols][None], y[cols][None])
            slack = (d1 - e[ri][:, None, None] - e[cols][None]).astype(np.float64)
            slack[cols[None] < ri[:, None, None] + 2] = np.inf
            bcrit = slack.min(axis=(0, 2))
            live = bcrit <= -1
            if not live.any():
                continue
            rbox = np.array([x[ri].min(), x[ri].max(), y[ri].min(), y[ri].max()], F)
            u = bcrit[live] + e[ri].max() + 5 + wmax[live]
            keep = _box_pass(rbox[None, :], wbox[live], u)
            assert keep.all(), (name, rows, i0, np.nonzero(~keep))
            tested += int(live.sum())
    assert tested > 0
