// All-pairs 2-opt move evaluation + argmin for one tour (sm_103a).
//
// Replaces kernel2opt / kernel2opt_extended (src/cuda/opt_kernel.cu:34-262,
// 273-627) and the inter-block atomicMin + spin mutex of :239-256.
//
// Candidate set (src/solvers/cpuSolver.cpp:188-230): pairs 1 <= i < j <= n-2
// of tour positions; with c = j + 1 (the reported j) the move deletes edges
// (i-1, i) and (c-1, c):
//     delta(i, c) = d(i, c) + d(i-1, c-1) - e[i] - e[c],   i+2 <= c <= n-1.
// Entry d(r, c) of the distance matrix serves pair (r, c) and pair
// (r+1, c+1), so a thread that owns R consecutive rows and walks columns
// computes R+1 distances per column for R pairs.
//
// Work split: the triangle is cut into tiles of (NW*32*R rows) x (cb
// columns); one CTA per tile.  The tile's columns [col0-1, col0+cb) are
// staged in shared memory with one bulk copy (TMA engine) and read back as
// broadcast 16-byte loads; each lane keeps its R+1 row points in registers.
//
// Exactness: the fast path uses approx_dist and a margin M bounding
// |exact delta - approximate delta|; a pair is re-evaluated with exact_dist
// only when approx < B + M (B = best exact delta known, <= -1).  Exact
// deltas <= B always pass, so the per-thread packed key
//     ((delta + 2^22) << 42) | (i << 21) | c
// ends up holding the lowest (delta, i, c), i.e. the reference CPU's choice
// (i ascending, j ascending, strict <).  Keys reduce by warp shuffle, shared
// memory, and one 64-bit atomicMin per CTA.
#include <atomic>

#include "logo_device.cuh"
#include "logo_internal.h"
#include "sweep_core.cuh"
#include "sweep_core3.cuh"
#include "sweep_core5.cuh"
#include "sweep_core6.cuh"
#include "sweep_core7.cuh"

namespace logo {

template <int R, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel(const OrderedCity* __restrict__ Q0,
                 const OrderedCity* __restrict__ Q1, uint32_t n,
                 const uint2* __restrict__ tiles, uint32_t cb, float margin,
                 DevState* st) {
    chain_wait();
    chain_release();
    extern __shared__ __align__(32) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* wbest = reinterpret_cast<uint64_t*>(smem_raw + 8);  // NW <= 8
    OrderedCity* cols = reinterpret_cast<OrderedCity*>(smem_raw + 80);

    if (*(volatile unsigned int*)&st->converged) return;
    const OrderedCity* Q = (*(volatile unsigned int*)&st->cur) ? Q1 : Q0;
    const uint2 tile = tiles[blockIdx.x];
    const uint32_t row0 = tile.x, col0 = tile.y;
    const uint32_t col_end = min(col0 + cb, n);
    const uint32_t ncols = col_end - col0 + 1;  // columns col0-1 .. col_end-1

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = ncols * (uint32_t)sizeof(OrderedCity);
        mbar_arrive_expect_tx(bar, bytes);
        bulk_g2s(cols, Q + (col0 - 1), bytes, bar);
    }

    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ib = row0 + (warp * 32 + lane) * R;
    uint64_t best = kNoMove;
    int B = -1;
    {
        const uint64_t gk = *(volatile unsigned long long*)&st->best_key;
        if (gk != kNoMove) B = min(B, key_delta(gk));
    }
    RowBlock<R> rb;
    load_rows<R>(rb, Q, ib, n);
    refresh_thresholds<R>(rb, Q, ib, n, B, margin);
    if (mbar_wait_bounded(bar, 0, &st->status))
        walk_columns<R>(rb, cols, col0 - 1, col0, col_end, ib, n, Q, margin, B, best);

    best = warp_min_u64(best);
    if (lane == 0) wbest[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t m = wbest[0];
#pragma unroll
        for (int w = 1; w < NW; ++w) m = wbest[w] < m ? wbest[w] : m;
        if (m != kNoMove) atomicMin(&st->best_key, (unsigned long long)m);
    }
}

// Fused two-stage variant (sweep_core5.cuh): the staged tile stays in shared
// memory for stages 2 and 3, beside a 16-byte (-x, -x, -y, -y) record per
// column for stage 1 and the largest edge of every 32-column window.
// Column groups of the fused screen: 64 / R columns (64 row entries per
// thread per branch; measured on GB300: G = 16 for 4-row blocks at n = 100k,
// 0.834 ms vs 0.850 with G = 8 and 0.899 ungrouped; G = 8 for 8-row blocks at
// n = 1M, 70.9 ms vs 71.7 with G = 16 and 74.2 with G = 4).
constexpr uint32_t kSweep5GroupMinN = 30000;
constexpr uint32_t kMaxTileRows = 2048;  // NW * 32 * R of the largest shapes, (16, 4) and (8, 8)

__host__ __device__ constexpr size_t sweep5_hot_offset(uint32_t cb) {
    return 96 + (size_t)(cb + 1) * sizeof(OrderedCity);
}
__host__ __device__ constexpr size_t sweep5_wmax_offset(uint32_t cb) {
    return sweep5_hot_offset(cb) + (size_t)(cb + 1) * sizeof(float4);
}

template <int R, int NW, int G>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel5(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                  uint32_t n, const uint2* __restrict__ tiles, uint32_t cb, float margin,
                  DevState* st) {
    chain_wait();
    chain_release();
    extern __shared__ __align__(32) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    OrderedCity* stage = reinterpret_cast<OrderedCity*>(smem_raw + 96);
    float4* hot = reinterpret_cast<float4*>(smem_raw + sweep5_hot_offset(cb));
    float* wmax = reinterpret_cast<float*>(smem_raw + sweep5_wmax_offset(cb));

    if (*(volatile unsigned int*)&st->converged) return;
    const OrderedCity* Q = (*(volatile unsigned int*)&st->cur) ? Q1 : Q0;
    const uint2 tile = tiles[blockIdx.x];
    const uint32_t row0 = tile.x, col0 = tile.y;
    const uint32_t col_end = min(col0 + cb, n);
    const uint32_t ncols = col_end - col0 + 1;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = ncols * (uint32_t)sizeof(OrderedCity);
        mbar_arrive_expect_tx(bar, bytes);
        bulk_g2s(stage, Q + (col0 - 1), bytes, bar);
    }
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ib = row0 + (warp * 32 + lane) * R;
    Best5 bs;
    bs.best = kNoMove;
    bs.B = -1;
    {
        const uint64_t gk = *(volatile unsigned long long*)&st->best_key;
        if (gk != kNoMove) bs.B = min(bs.B, key_delta(gk));
    }
    bs.G = bs.B;
    bs.busy = false;
    bs.M = margin;
    RowBlock5<R> rb;
    load_rows5<R>(rb, Q, ib, n);
    refresh5<R>(rb, Q, ib, n, bs.B);
    const bool staged = mbar_wait_bounded(bar, 0, &st->status);
    const uint32_t nwin = (col_end - col0 + kWin5 - 1) / kWin5;
    if (staged) {
        for (uint32_t k = threadIdx.x; k < ncols; k += NW * 32) {
            const OrderedCity q = stage[k];
            hot[k] = make_float4(-q.x, -q.x, -q.y, -q.y);
        }
        for (uint32_t w = threadIdx.x; w < nwin; w += NW * 32) {
            const uint32_t a = 1 + w * kWin5, b = min(a + kWin5, ncols);
            float m = 0.f;
            for (uint32_t k = a; k < b; ++k) m = fmaxf(m, stage[k].e);
            wmax[w] = m;
        }
    }
    __syncthreads();
    if (staged)
        walk_columns5<R, G>(rb, hot, stage, col0 - 1, wmax, col0, col0, col_end, ib, n, st, bs);

    // per-warp result: no CTA barrier at the end; most warps found nothing
    // (their B was already the sweep's best) and skip the atomic
    const uint64_t best = warp_min_u64(bs.best);
    if (lane == 0 && best != kNoMove) atomicMin(&st->best_key, (unsigned long long)best);
}

// Local-coordinate expanded variant (sweep_core6.cuh): the staged tile stays
// in shared memory for stages 2 and 3, beside three float arrays (p, q, C of
// every column relative to the tile's origin, read as float4 by stage 1) and
// the largest edge of every 32-column window.
__host__ __device__ constexpr size_t sweep6_cols4(uint32_t cb) { return (cb + 3) & ~(size_t)3; }
__host__ __device__ constexpr size_t sweep6_cx_offset(uint32_t cb) {
    return 96 + (size_t)(cb + 1) * sizeof(OrderedCity);
}
__host__ __device__ constexpr size_t sweep6_wmax_offset(uint32_t cb) {
    return sweep6_cx_offset(cb) + 3 * sweep6_cols4(cb) * sizeof(float);
}
template <int R, int NW, int G>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel6(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                  uint32_t n, const uint2* __restrict__ tiles, uint32_t cb, float margin,
                  DevState* st) {
    chain_wait();
    chain_release();
    extern __shared__ __align__(32) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    OrderedCity* stage = reinterpret_cast<OrderedCity*>(smem_raw + 96);
    float* cx = reinterpret_cast<float*>(smem_raw + sweep6_cx_offset(cb));
    float* cy = cx + sweep6_cols4(cb);
    float* cc = cy + sweep6_cols4(cb);
    float* wmax = reinterpret_cast<float*>(smem_raw + sweep6_wmax_offset(cb));

    if (*(volatile unsigned int*)&st->converged) return;
    const OrderedCity* Q = (*(volatile unsigned int*)&st->cur) ? Q1 : Q0;
    const uint2 tile = tiles[blockIdx.x];
    const uint32_t row0 = tile.x, col0 = tile.y;
    const uint32_t col_end = min(col0 + cb, n);
    const uint32_t ncols = col_end - col0 + 1;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = ncols * (uint32_t)sizeof(OrderedCity);
        mbar_arrive_expect_tx(bar, bytes);
        bulk_g2s(stage, Q + (col0 - 1), bytes, bar);
    }
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ib = row0 + (warp * 32 + lane) * R;
    Best5 bs;
    bs.best = kNoMove;
    bs.B = -1;
    {
        const uint64_t gk = *(volatile unsigned long long*)&st->best_key;
        if (gk != kNoMove) bs.B = min(bs.B, key_delta(gk));
    }
    bs.G = bs.B;
    bs.busy = false;
    bs.M = margin;
    const OrderedCity origin = Q[row0];  // same for every thread of the tile
    RowBlock6<R> rb;
    load_rows6<R>(rb, Q, ib, n, origin.x, origin.y);
    refresh6<R>(rb, Q, ib, n, bs.B);
    const bool staged = mbar_wait_bounded(bar, 0, &st->status);
    const uint32_t nwin = (col_end - col0 + kWin6 - 1) / kWin6;
    if (staged) {
        for (uint32_t k = threadIdx.x + 1; k < ncols; k += NW * 32) {
            const OrderedCity q = stage[k];
            const float p = __fsub_rn(q.x, origin.x), qq = __fsub_rn(q.y, origin.y);
            cx[k - 1] = p;
            cy[k - 1] = qq;
            cc[k - 1] = __fmaf_rn(qq, qq, __fmul_rn(p, p));
        }
        // window maxima: one warp per window, one lane per column
        static_assert(kWin6 == 32, "one lane per column of a window");
        const uint32_t lane6 = threadIdx.x & 31;
        for (uint32_t w = threadIdx.x >> 5; w < nwin; w += NW) {
            const uint32_t k = 1 + w * kWin6 + lane6;
            float m = k < ncols ? stage[k].e : 0.f;
            for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane6 == 0) wmax[w] = m;
        }
    }
    __syncthreads();
    if (staged) {
        const ColTile6 t{cx, cy, cc, stage};
        walk_columns6<R, G, false>(rb, t, wmax, nullptr, 0u, col0, col0, col_end, ib, n, st, bs);
    }

    const uint64_t best = warp_min_u64(bs.best);
    if (lane == 0 && best != kNoMove) atomicMin(&st->best_key, (unsigned long long)best);
}

// Boxed variant, pass 1: for every window of 32 columns (columns 3 + 32 g
// .. 3 + 32 g + 31, below n) the bounding box of its coordinates and its
// largest edge, and the same for every window of 32 rows (rows 1 + 32 g ..,
// only rows with pairs, i + 3 <= n; a window without such rows gets an
// empty box and -3e7), one warp per window, together with the seed of the
// sweep's bound (seed_position for the warp's 32 positions).  Also clears
// the work-list counters of pass 2.
__device__ __forceinline__ void window_reduce(float& m, float& x0, float& x1, float& y0,
                                              float& y1) {
    for (int o = 16; o; o >>= 1) {
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    }
}

// Seed of the sweep's bound at tour position i: for each of the
// kSeedNeighbours nearest neighbours v of its city (at position p = pos[v]),
// the two pairs whose move creates the short edge (i, p): (a, b) =
// (min, max) of (i, p), whose delta has d(a, b) = d(i, p) as its first term,
// and (a + 1, b + 1), which has it as its second.  Their exact deltas are
// real pairs of this sweep, so the best of them is a valid starting bound:
// the sweep's best delta is at most that, and the tile filter and the boxed
// kernel prune with it from the start instead of with -1.  The lowest key
// goes to st->best_key, where it competes with every other pair, so the
// chosen move is still the exact lowest (delta, i, c).  Any p the position
// array gives names a real pair, so a stale entry costs seed quality only.
__device__ __forceinline__ void seed_position(const OrderedCity* __restrict__ Q,
                                              const uint32_t* __restrict__ R,
                                              const uint32_t* __restrict__ pos,
                                              const uint32_t* __restrict__ nbr, uint32_t n,
                                              uint32_t i, uint64_t& best) {
    constexpr uint32_t K = kSeedNeighbours;
    // every load of the position's candidates is issued before any is used
    const uint32_t t = min(R[i], n - 1);
    const OrderedCity qi = Q[i], qim = Q[i >= 1 ? i - 1 : 0], qip = Q[min(i + 1, n - 1)];
    uint32_t p[K];
#pragma unroll
    for (uint32_t k = 0; k < K; ++k) p[k] = nbr[(size_t)t * K + k];
#pragma unroll
    for (uint32_t k = 0; k < K; ++k) p[k] = min(pos[min(p[k], n - 1)], n - 1);
    OrderedCity qp[K], qpm[K], qpp[K];
#pragma unroll
    for (uint32_t k = 0; k < K; ++k) {
        qp[k] = Q[p[k]];
        qpm[k] = Q[p[k] >= 1 ? p[k] - 1 : 0];
        qpp[k] = Q[min(p[k] + 1, n - 1)];
    }
#pragma unroll
    for (uint32_t k = 0; k < K; ++k) {
        const uint32_t a = min(i, p[k]), b = max(i, p[k]);
        if (b < a + 2) continue;  // also p == i
        const int D = exact_dist(qi.x, qi.y, qp[k].x, qp[k].y);
        const int ee = (int)qi.e + (int)qp[k].e;
        if (a >= 1) {
            // pair (a, b): d(a, b) + d(a - 1, b - 1) - e[a] - e[b]
            const int delta = D + exact_dist(qim.x, qim.y, qpm[k].x, qpm[k].y) - ee;
            if (delta < 0) {
                const uint64_t key = pack_key(delta, a, b);
                best = key < best ? key : best;
            }
        }
        if (b + 1 <= n - 1) {
            // pair (a + 1, b + 1): d(a + 1, b + 1) + d(a, b) - e[a + 1] - e[b + 1]
            const int delta = exact_dist(qip.x, qip.y, qpp[k].x, qpp[k].y) + D -
                              (int)qip.e - (int)qpp[k].e;
            if (delta < 0) {
                const uint64_t key = pack_key(delta, a + 1, b + 1);
                best = key < best ? key : best;
            }
        }
    }
}

__global__ void __launch_bounds__(256)
    window_seed_kernel(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                       const uint32_t* __restrict__ R0, const uint32_t* __restrict__ R1,
                       const uint32_t* __restrict__ pos, const uint32_t* __restrict__ nbr,
                       uint32_t n, float4* __restrict__ wbox, float* __restrict__ wmax,
                       float4* __restrict__ rbox, float* __restrict__ rmax,
                       uint32_t* __restrict__ workctl, uint32_t stride, DevState* st) {
    chain_wait();
    chain_release();
    if (*(volatile unsigned int*)&st->converged) return;
    if (blockIdx.x == 0 && threadIdx.x < 3) workctl[threadIdx.x] = 0u;
    const bool cur = *(volatile unsigned int*)&st->cur;
    const OrderedCity* Q = cur ? Q1 : Q0;
    const uint32_t* R = cur ? R1 : R0;
    const uint32_t g = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (g < sweep_windows(n)) {  // whole warps
        const uint32_t c = 3 + g * kWin6 + lane;
        const bool in = c < n;
        const OrderedCity q = Q[in ? c : n - 1];
        float m = in ? q.e : 0.f;
        float x0 = in ? q.x : FLT_MAX, x1 = in ? q.x : -FLT_MAX;
        float y0 = in ? q.y : FLT_MAX, y1 = in ? q.y : -FLT_MAX;
        window_reduce(m, x0, x1, y0, y1);
        if (lane == 0) {
            wbox[g] = make_float4(x0, x1, y0, y1);
            wmax[g] = m;
        }
    }
    if (g < sweep_row_windows(n)) {
        const uint32_t i = 1 + g * kWin6 + lane;
        const bool in = i + 3 <= n;
        const OrderedCity q = Q[in ? i : 1];
        float m = in ? q.e : -3.0e7f;
        float x0 = in ? q.x : FLT_MAX, x1 = in ? q.x : -FLT_MAX;
        float y0 = in ? q.y : FLT_MAX, y1 = in ? q.y : -FLT_MAX;
        window_reduce(m, x0, x1, y0, y1);
        if (lane == 0) {
            rbox[g] = make_float4(x0, x1, y0, y1);
            rmax[g] = m;
        }
    }
    // the seed: positions 3 + stride * (32 g + lane), and 0, 1, 2 in the
    // first warp
    uint64_t best = kNoMove;
    const uint32_t i = 3 + stride * (g * kWin6 + lane);
    if (i < n) seed_position(Q, R, pos, nbr, n, i, best);
    if (g == 0 && lane < 3 && lane < n) seed_position(Q, R, pos, nbr, n, lane, best);
    best = warp_min_u64(best);
    if (lane == 0 && best != kNoMove) atomicMin(&st->best_key, (unsigned long long)best);
}

// Boxed variant, pass 2: gridDim.y CTAs per row block (the rows of one tile
// row, rows_per_tile of them from row0 = 1 + rows_per_tile * blockIdx.x).
// The block's row-window statistics go to shared memory; each warp then
// takes 32 consecutive column windows of the block at a time (lane = column
// window, 32 / (cb / 32) tiles per step; the CTAs of a row block split its
// steps) and tests them against every row window with B = the seed pass's
// best delta, or -1 (the largest best delta a sweep can end with) if it
// found none (box_gap_pass with u = B + E_r + 5 + E_c, which bounds every
// V + 5 of those pairs).  Tiles with a passing pair are appended to the work list as
// (row0, col0, mask of their column windows that passed).  The tiles are
// the ones the tile list holds: columns from row0 + 2 to n - 1 in steps of
// cb.
// Steps (32 column windows each) per filter warp on the longest row block:
// fewer, longer-lived CTAs share the per-CTA start (the bound, the row
// block's windows and their union) over several steps (measured on GB300:
// n = 100k sweep of the benchmark's states 0.0645 ms with 4, 0.0688 with 1,
// 0.0655 with 8; n = 1M random tour 0.208 ms with 8, 0.232 with 4).
__host__ __device__ constexpr uint32_t filter_steps(uint32_t n) { return n >= 300000 ? 8u : 4u; }

// Positions the seed pass evaluates: every one, or every stride-th on the
// largest tours, where the pass is most of a sweep and a bound from a
// sample of the positions prunes about as well (measured on GB300, n = 1M
// uniform random tour: stride 1, 2, 3, 4, 8 -> 0.203, 0.158, 0.134, 0.129,
// 0.260 ms per sweep).
#ifndef LOGO_SEED_SPARSE
#define LOGO_SEED_SPARSE 4
#endif
__host__ __device__ constexpr uint32_t seed_stride(uint32_t n) {
    return n >= 500000 ? (uint32_t)LOGO_SEED_SPARSE : 1u;
}

// Tiles the filter lists first: those whose rows and columns are close
// along the tour (the tile meets its row block's own positions), which on
// tours built or improved by local moves are close in space too, so most of
// their rows stay open and they are the longest items; starting them first
// keeps them off the end of the sweep.  Every other tile is listed from the
// end of the array.
__device__ __forceinline__ bool front_tile(uint32_t row0, uint32_t col0, uint32_t rows_per_tile,
                                           uint32_t mask, uint32_t wpt) {
    (void)mask;
    (void)wpt;
    return col0 < row0 + 2 + rows_per_tile;
}

__global__ void __launch_bounds__(256)
    tile_filter_kernel(uint32_t n, uint32_t rows_per_tile, uint32_t cb,
                       const float4* __restrict__ wbox, const float* __restrict__ wmax,
                       const float4* __restrict__ rbox, const float* __restrict__ rmax,
                       uint4* __restrict__ work, uint32_t cap, uint32_t* __restrict__ workctl,
                       DevState* st) {
    chain_wait();
    chain_release();
    __shared__ float4 srb[kMaxTileRows / kWin6];
    __shared__ float sre[kMaxTileRows / kWin6];
    if (*(volatile unsigned int*)&st->converged) return;
    // B: the seed pass's best delta (a real pair of this sweep), else -1
    int B = -1;
    {
        const uint64_t gk = *(volatile unsigned long long*)&st->best_key;
        if (gk != kNoMove) B = min(B, key_delta(gk));
    }
    const float b5 = (float)(B + 5);
    const uint32_t row0 = 1 + blockIdx.x * rows_per_tile;
    const uint32_t ntiles = (n - row0 - 2 + cb - 1) / cb;  // columns row0 + 2 .. n - 1
    const uint32_t wpt = cb / kWin6;                       // windows per tile (cb % 32 == 0)
    const uint32_t tps = 32u / wpt;                        // tiles per step
    if (blockIdx.y * 8 * tps >= ntiles) return;            // the whole CTA
    const uint32_t row_end = min(row0 + rows_per_tile, n - 2);  // rows i + 3 <= n
    const uint32_t nrw = (row_end - row0 + kWin6 - 1) / kWin6;
    const uint32_t rw0 = (row0 - 1) / kWin6;
    __shared__ float4 sub;  // the whole row block: union of its row windows' boxes
    __shared__ float sue;   // and their largest edge
    for (uint32_t r = threadIdx.x; r < nrw; r += blockDim.x) {
        srb[r] = rbox[rw0 + r];
        sre[r] = rmax[rw0 + r];
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        float m = -3.0e7f, x0 = FLT_MAX, x1 = -FLT_MAX, y0 = FLT_MAX, y1 = -FLT_MAX;
        for (uint32_t r = lane; r < nrw; r += 32) {
            const float4 b = srb[r];
            m = fmaxf(m, sre[r]);
            x0 = fminf(x0, b.x);
            x1 = fmaxf(x1, b.y);
            y0 = fminf(y0, b.z);
            y1 = fmaxf(y1, b.w);
        }
        window_reduce(m, x0, x1, y0, y1);
        if (lane == 0) {
            sub = make_float4(x0, x1, y0, y1);
            sue = m;
        }
    }
    __syncthreads();
    const uint32_t col_start = row0 + 2;
    for (uint32_t t0 = (blockIdx.y * 8 + warp) * tps; t0 < ntiles; t0 += gridDim.y * 8 * tps) {
        const uint32_t tk = t0 + lane / wpt;
        const uint32_t col = col_start + tk * cb + (lane % wpt) * kWin6;  // window start
        bool any = false;
        if (tk < ntiles && lane < tps * wpt && col < n) {
            const uint32_t cw = (col - 3) / kWin6;
            const float4 cbx = wbox[cw];
            const float ce = wmax[cw];
            const uint32_t last_col = min(col + kWin6, n) - 1;
            // the block test first: no row window passes unless the union does
            const bool block = box_gap_pass(sub, cbx, (sue + b5) + ce);
            for (uint32_t r = 0; block && r < nrw; ++r) {
                if (last_col < row0 + r * kWin6 + 2) break;  // no pair c >= i + 2 from here on
                if (box_gap_pass(srb[r], cbx, (sre[r] + b5) + ce)) {
                    any = true;
                    break;
                }
            }
        }
        const uint32_t votes = __ballot_sync(0xffffffffu, any);
        if (lane < tps && t0 + lane < ntiles) {
            const uint32_t mask =
                (votes >> (lane * wpt)) & (wpt == 32 ? 0xffffffffu : ((1u << wpt) - 1u));
            if (mask) {
                const uint32_t col0 = col_start + (t0 + lane) * cb;
                const uint32_t k = front_tile(row0, col0, rows_per_tile, mask, wpt)
                                       ? atomicAdd(&workctl[0], 1u)
                                       : cap - 1u - atomicAdd(&workctl[2], 1u);
                work[k] = make_uint4(row0, col0, mask, 0u);
            }
        }
    }
}

// Boxed variant, pass 3 (LOGO_SWEEP_BOXED, sweep_core7.cuh): a persistent
// grid takes the work list's tiles one at a time.  Per tile, each thread
// loads its R rows and, for every window the filter kept, runs the block
// test and the one-row tests with its current B; what passes goes into a
// queue of units (thread, window, rows) in shared memory.  Only tiles with
// units stage their columns (one bulk copy of the range the units touch).
// A tile with few units has its warps take them round robin, one lane per
// column, so the rare open blocks are spread over the CTA and no lane idles
// on a closed one.  A tile whose units would keep most lanes busy is walked
// the way sweep_kernel6 walks a tile instead, every thread over its open
// windows with the local-coordinate screen, which is cheaper per pair when
// most lanes have work: a warp walks for as long as its busiest lane, each
// open window costing about as much as kWalkRows open rows of units, so the
// tile is walked when its open rows exceed kWalkRows x R x (sum over warps
// of the busiest lane's open windows).
// Tile columns start at 3 + 32k (tile widths are multiples of 32) and rows
// at 1 + 32k, so tile window w is window (col0 - 3) / 32 + w of pass 1.  B
// carries over from tile to tile, is tightened with the sweep's shared best
// at every claim and shared within a warp after every unit.  A CTA claims
// its next item only when it is free (claiming ahead left items reserved by
// busy CTAs while others ran out).
struct BoxedSlot {
    uint32_t idx;
    uint32_t need;            // windows the units touch
    unsigned long long best;  // the sweep's best key when the item was claimed
    uint4 item;               // row0, col0, column-window mask
    uint32_t units;           // units queued
    uint32_t walk;            // sum over warps of the most windows one lane opened
    uint32_t rows;            // open rows over all units
};
// Open rows of units that take as long as walking one window per row of a
// thread (measured on GB300, n = 100k, (4, 4, 128) tiles: NN start tour
// 0.090 ms and its local optimum 0.109 ms with 16; 0.093 / 0.126 with 8;
// 0.135 / 0.107 with 32; walking every tile with a unit 0.094 / 0.130).
constexpr uint32_t kWalkRows = 16;
constexpr size_t kBoxedStageOffset = 96;
__host__ __device__ constexpr size_t boxed_queue_offset(uint32_t cb) {
    return kBoxedStageOffset + (((size_t)cb + 1) * sizeof(OrderedCity) + 15) / 16 * 16;
}
__host__ __device__ constexpr size_t boxed_cx_offset(uint32_t cb, int NW) {
    return boxed_queue_offset(cb) + (size_t)NW * 32 * (cb / kWin7) * sizeof(uint32_t);
}
__host__ __device__ constexpr size_t boxed_smem_bytes(uint32_t cb, int NW) {
    return boxed_cx_offset(cb, NW) + 3 * sweep6_cols4(cb) * sizeof(float);
}

// Resident CTAs per SM the boxed kernel is compiled for (register budget:
// 4-row threads at 96 registers, 8-row threads at 128).
constexpr int boxed_min_blocks(int R, int NW) {
    return R == 4 ? (NW == 2 ? 10 : NW == 4 ? 5 : 2) : R == 8 ? (NW == 8 ? 2 : 4) : 1;
}

__device__ __forceinline__ int warp_min_int(int v) {
    for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <int R, int NW>
__global__ void __launch_bounds__(NW * 32, boxed_min_blocks(R, NW))
    sweep_boxed_kernel(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                       uint32_t n, uint32_t cb, const float4* __restrict__ gbox,
                       const float* __restrict__ gmax, const uint4* __restrict__ work,
                       uint32_t cap, float margin, uint32_t* __restrict__ workctl,
                       DevState* st) {
    chain_wait();
    chain_release();
    static_assert(R <= 16 && NW * 32 <= 256, "unit encoding: 8-bit thread, 16-bit rows");
    constexpr int G = (128 / R) < 32 ? (128 / R) : 32;
    extern __shared__ __align__(32) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    BoxedSlot* slot = reinterpret_cast<BoxedSlot*>(smem_raw + 16);  // 48 bytes
    OrderedCity* stage = reinterpret_cast<OrderedCity*>(smem_raw + kBoxedStageOffset);
    uint32_t* queue = reinterpret_cast<uint32_t*>(smem_raw + boxed_queue_offset(cb));
    __shared__ float4 sbox[kWin7];  // the claimed tile's window statistics
    __shared__ float smax[kWin7];
    float* cx = reinterpret_cast<float*>(smem_raw + boxed_cx_offset(cb, NW));
    float* cy = cx + sweep6_cols4(cb);
    float* cc = cy + sweep6_cols4(cb);

    if (*(volatile unsigned int*)&st->converged) return;
    const OrderedCity* Q = (*(volatile unsigned int*)&st->cur) ? Q1 : Q0;
    // the filter's list: items [0, front) from the start, the rest from the end
    const uint32_t front = workctl[0];
    const uint32_t items = front + workctl[2];
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Best5 bs;
    bs.best = kNoMove;
    bs.B = -1;
    {
        const uint64_t gk = *(volatile unsigned long long*)&st->best_key;
        if (gk != kNoMove) bs.B = min(bs.B, key_delta(gk));
    }
    bs.G = bs.B;
    bs.M = margin;
    uint32_t parity = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t idx = atomicAdd(&workctl[1], 1u);
            slot->idx = idx;
            slot->need = 0u;
            slot->units = 0u;
            slot->walk = 0u;
            slot->rows = 0u;
            slot->best = *(volatile unsigned long long*)&st->best_key;
            if (idx < items) slot->item = work[idx < front ? idx : cap - 1u - (idx - front)];
        }
        __syncthreads();  // the slot is ready (the previous tile ended in a barrier)
        if (slot->idx >= items) break;
        const uint4 item = slot->item;
        {
            const uint64_t gk = slot->best;
            if (gk != kNoMove) {
                const int g = key_delta(gk);
                bs.B = min(bs.B, g);
                bs.G = min(bs.G, g);
            }
        }
        const uint32_t row0 = item.x, col0 = item.y;
        const uint32_t col_end = min(col0 + cb, n);
        const float4* tbox = gbox + (col0 - 3) / kWin7;
        const float* tmax = gmax + (col0 - 3) / kWin7;
        const uint32_t ib = row0 + threadIdx.x * R;
        // the tile's window statistics, all loaded at once (loading them
        // inside the window loop cost one round trip each)
        if (threadIdx.x < kWin7 && ((item.z >> threadIdx.x) & 1u)) {
            sbox[threadIdx.x] = tbox[threadIdx.x];
            smax[threadIdx.x] = tmax[threadIdx.x];
        }
        __syncthreads();
        uint32_t open = 0;  // windows in which some row of this thread is open
        uint32_t rows = 0;  // open rows over this thread's units
        if (ib + 3 <= n) {
            RowBlock7<R> rb;
            load_rows7<R>(rb, Q, ib, n, bs.B);
            for (uint32_t m = item.z; m; m &= m - 1) {
                const uint32_t w = __ffs(m) - 1;
                if (col0 + (w + 1) * kWin7 <= ib + 2) continue;  // left of the first pair
                const uint32_t rm = rows_open7<R>(rb, sbox[w], smax[w]);
                if (rm) {
                    queue[atomicAdd(&slot->units, 1u)] = (threadIdx.x << 24) | (w << 16) | rm;
                    open |= 1u << w;
                    rows += __popc(rm);
                }
            }
            if (open) atomicOr(&slot->need, open);
        }
        {
            const uint32_t busiest = __reduce_max_sync(0xffffffffu, (uint32_t)__popc(open));
            const uint32_t wrows = __reduce_add_sync(0xffffffffu, rows);
            if (lane == 0 && busiest) {
                atomicAdd(&slot->walk, busiest);
                atomicAdd(&slot->rows, wrows);
            }
        }
        __syncthreads();
        const uint32_t units = slot->units, all = slot->need;
        if (units) {  // the same for every thread
            const uint32_t wlo = __ffs(all) - 1, whi = 31 - __clz(all);
            // stage[k] = column col0 - 1 + k for k in [k0, k1)
            const uint32_t k0 = wlo * kWin7, k1 = min((whi + 1) * kWin7, col_end - col0) + 1;
            if (threadIdx.x == 0) {
                const uint32_t bytes = (k1 - k0) * (uint32_t)sizeof(OrderedCity);
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(bar, bytes);
                bulk_g2s(stage + k0, Q + (col0 - 1 + k0), bytes, bar);
            }
            const bool ok = mbar_wait_bounded(bar, parity, &st->status);
            parity ^= 1u;
            if (slot->rows > kWalkRows * R * slot->walk) {  // the same for every thread
                const OrderedCity origin = Q[row0];
                if (ok) {
                    for (uint32_t k = k0 + 1 + threadIdx.x; k < k1; k += NW * 32) {
                        const OrderedCity q = stage[k];
                        const float p = __fsub_rn(q.x, origin.x), qq = __fsub_rn(q.y, origin.y);
                        cx[k - 1] = p;
                        cy[k - 1] = qq;
                        cc[k - 1] = __fmaf_rn(qq, qq, __fmul_rn(p, p));
                    }
                }
                // a copy that did not arrive ends the CTA's work (status has the timeout)
                if (__syncthreads_or(!ok)) break;
                if (open) {
                    RowBlock6<R> rb;
                    load_rows6<R>(rb, Q, ib, n, origin.x, origin.y);
                    refresh6<R>(rb, Q, ib, n, bs.B);
                    const ColTile6 t{cx, cy, cc, stage};
                    walk_columns6<R, G, true>(rb, t, tmax, tbox, open, col0, col0, col_end, ib, n,
                                              st, bs);
                }
            } else {
                if (__syncthreads_or(!ok)) break;
                for (uint32_t u = warp; u < units; u += NW) {
                    const uint32_t e = queue[u];
                    const uint32_t uib = row0 + (e >> 24) * R, w = (e >> 16) & 0xffu;
                    const uint32_t c = col0 + w * kWin7 + lane;
                    if (c < col_end)
                        unit7<R>(Q, stage, col0, c, uib, e & 0xffffu, n, bs.M, bs.B, bs.best);
                    bs.B = warp_min_int(bs.B);
                    if (bs.B < bs.G) {  // publish the warp's best
                        const uint64_t k = warp_min_u64(bs.best);
                        if (lane == 0) atomicMin(&st->best_key, (unsigned long long)k);
                        bs.G = bs.B;
                    }
                }
            }
        }
        __syncthreads();  // every thread has read the slot, the queue and the stage
    }

    const uint64_t k = warp_min_u64(bs.best);
    if (lane == 0 && k != kNoMove) atomicMin(&st->best_key, (unsigned long long)k);
}

size_t sweep_smem_bytes(uint32_t cb) { return 80 + (size_t)(cb + 1) * sizeof(OrderedCity); }

// The dynamic shared-memory limit is a property of the kernel, shared by
// every context in the process: it is always set for the largest tile a
// context may choose (4096 columns), never for this context's own tile, so
// that contexts created later cannot lower it under another one's launch.
constexpr uint32_t kMaxTileCols = 4096;
constexpr uint32_t kMaxBoxedCols = 1024;  // one mask bit per 32-column window
inline int attr_bytes(size_t smem) { return (int)(smem > 48 * 1024 ? smem : 48 * 1024); }

size_t sweep5_smem_bytes(uint32_t cb) {
    return sweep5_wmax_offset(cb) + ((size_t)cb / kWin5 + 2) * sizeof(float);
}

template <int R, int NW, int G>
static cudaError_t launch_sweep5_g(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = sweep5_smem_bytes(L.cb);
    if (prepare) {
        return cudaFuncSetAttribute(sweep_kernel5<R, NW, G>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    attr_bytes(sweep5_smem_bytes(kMaxTileCols)));
    }
    return launch_chained(sweep_kernel5<R, NW, G>, L.ntiles, NW * 32, smem, s, L.Q0, L.Q1, L.n,
                          L.tiles, L.cb, L.margin, L.st);
}

// Column grouping of the fused screen: on large tours few columns pass and
// grouping saves branches; on smaller ones (every CTA starts before a tight
// best is known) the per-column walk is faster.
template <int R, int NW>
static cudaError_t launch_sweep5_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    constexpr int G = 64 / R;
    if (prepare) {
        const cudaError_t e = launch_sweep5_g<R, NW, 1>(L, s, true);
        return e != cudaSuccess ? e : launch_sweep5_g<R, NW, G>(L, s, true);
    }
    return L.n >= kSweep5GroupMinN ? launch_sweep5_g<R, NW, G>(L, s, false)
                                   : launch_sweep5_g<R, NW, 1>(L, s, false);
}

size_t sweep6_smem_bytes(uint32_t cb) {
    return sweep6_wmax_offset(cb) + ((size_t)cb / kWin6 + 2) * sizeof(float);
}

template <int R, int NW, int G>
static cudaError_t launch_sweep6_g(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = sweep6_smem_bytes(L.cb);
    if (prepare) {
        return cudaFuncSetAttribute(sweep_kernel6<R, NW, G>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    attr_bytes(sweep6_smem_bytes(kMaxTileCols)));
    }
    return launch_chained(sweep_kernel6<R, NW, G>, L.ntiles, NW * 32, smem, s, L.Q0, L.Q1, L.n,
                          L.tiles, L.cb, L.margin, L.st);
}

// Boxed variant: window statistics with the near-neighbour seed, tile
// filter, persistent sweep (one CTA per resident slot).
template <int R, int NW>
static cudaError_t launch_boxed_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = boxed_smem_bytes(L.cb, NW);
    if (prepare) {
        return cudaFuncSetAttribute(sweep_boxed_kernel<R, NW>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    attr_bytes(boxed_smem_bytes(kMaxBoxedCols, NW)));
    }
    // resident CTAs of this shape per device and tile width, computed once
    static std::atomic<uint32_t> cached[64][kMaxBoxedCols / kWin7 + 1];
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    std::atomic<uint32_t>& slot = cached[(unsigned)device % 64][L.cb / kWin7];
    uint32_t resident = slot.load(std::memory_order_relaxed);
    if (resident == 0) {
        int sms = 0, per_sm = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_boxed_kernel<R, NW>,
                                                              NW * 32, smem);
        if (e != cudaSuccess) return e;
        resident = (uint32_t)(per_sm > 0 ? per_sm : 1) * (uint32_t)sms;
        slot.store(resident, std::memory_order_relaxed);
    }
    const uint32_t grid = L.ntiles < resident ? L.ntiles : resident;
    const uint32_t nwin = max(sweep_windows(L.n), sweep_row_windows(L.n));
    e = launch_chained(window_seed_kernel, (nwin + 7) / 8, 256, 0, s, L.Q0, L.Q1, L.R0, L.R1,
                       L.pos, L.nbr, L.n, L.wbox, L.wmax, L.rbox, L.rmax, L.workctl,
                       seed_stride(L.n), L.st);
    if (e != cudaSuccess) return e;
    const uint32_t rows_per_tile = (uint32_t)(NW * 32 * R);
    const uint32_t row_blocks = (L.n - 4) / rows_per_tile + 1;  // row0 + 3 <= n
    // CTAs per row block: filter_steps(n) steps per warp for the longest row (block 0)
    const uint32_t steps = ((L.n - 3 + L.cb - 1) / L.cb + 32 / (L.cb / 32) - 1) / (32 / (L.cb / 32));
    const uint32_t fs = filter_steps(L.n);
    const dim3 fgrid(row_blocks, (steps + 8 * fs - 1) / (8 * fs));
    e = launch_chained(tile_filter_kernel, fgrid, 256, 0, s, L.n, rows_per_tile, L.cb, L.wbox,
                       L.wmax, L.rbox, L.rmax, L.work, L.ntiles, L.workctl, L.st);
    if (e != cudaSuccess) return e;
    return launch_chained(sweep_boxed_kernel<R, NW>, grid, NW * 32, smem, s, L.Q0, L.Q1, L.n,
                          L.cb, L.wbox, L.wmax, L.work, L.ntiles, L.margin, L.workctl, L.st);
}

// Column groups of the local-coordinate screen: 128 / R columns per branch
// (measured on GB300 with 4-row blocks: n = 100k 0.631 ms with 32 columns vs
// 0.641 with 16; n = 1M 54.7 ms vs 55.5), 4 below kSweep5GroupMinN cities.
template <int R, int NW>
static cudaError_t launch_sweep6_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    constexpr int G = (128 / R) < 32 ? (128 / R) : 32;
    if (prepare) {
        const cudaError_t e = launch_sweep6_g<R, NW, 4>(L, s, true);
        return e != cudaSuccess ? e : launch_sweep6_g<R, NW, G>(L, s, true);
    }
    return L.n >= kSweep5GroupMinN ? launch_sweep6_g<R, NW, G>(L, s, false)
                                   : launch_sweep6_g<R, NW, 4>(L, s, false);
}

template <int R, int NW>
static cudaError_t launch_sweep_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = sweep_smem_bytes(L.cb);
    if (prepare) {
        // opt-in above 48 KB; called once per shape, outside stream capture
        return cudaFuncSetAttribute(sweep_kernel<R, NW>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    attr_bytes(sweep_smem_bytes(kMaxTileCols)));
    }
    return launch_chained(sweep_kernel<R, NW>, L.ntiles, NW * 32, smem, s, L.Q0, L.Q1, L.n,
                          L.tiles, L.cb, L.margin, L.st);
}

static cudaError_t dispatch_sweep(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    if (L.variant == 6) {
        switch (L.R * 100 + L.NW) {
            case 402: return launch_boxed_t<4, 2>(L, s, prepare);
            case 404: return launch_boxed_t<4, 4>(L, s, prepare);
            case 408: return launch_boxed_t<4, 8>(L, s, prepare);
            case 804: return launch_boxed_t<8, 4>(L, s, prepare);
            case 808: return launch_boxed_t<8, 8>(L, s, prepare);
            case 1604: return launch_boxed_t<16, 4>(L, s, prepare);
            default: return cudaErrorInvalidValue;
        }
    }
    if (L.variant == 5) {
        switch (L.R * 100 + L.NW) {
            case 402: return launch_sweep6_t<4, 2>(L, s, prepare);
            case 404: return launch_sweep6_t<4, 4>(L, s, prepare);
            case 408: return launch_sweep6_t<4, 8>(L, s, prepare);
            case 804: return launch_sweep6_t<8, 4>(L, s, prepare);
            case 808: return launch_sweep6_t<8, 8>(L, s, prepare);
            case 1604: return launch_sweep6_t<16, 4>(L, s, prepare);
            default: return cudaErrorInvalidValue;
        }
    }
    if (L.variant == 4) {
        switch (L.R * 100 + L.NW) {
            case 402: return launch_sweep5_t<4, 2>(L, s, prepare);
            case 404: return launch_sweep5_t<4, 4>(L, s, prepare);
            case 408: return launch_sweep5_t<4, 8>(L, s, prepare);
            case 802: return launch_sweep5_t<8, 2>(L, s, prepare);
            case 804: return launch_sweep5_t<8, 4>(L, s, prepare);
            case 808: return launch_sweep5_t<8, 8>(L, s, prepare);
            case 1604: return launch_sweep5_t<16, 4>(L, s, prepare);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (L.R * 100 + L.NW) {
        case 202: return launch_sweep_t<2, 2>(L, s, prepare);
        case 204: return launch_sweep_t<2, 4>(L, s, prepare);
        case 402: return launch_sweep_t<4, 2>(L, s, prepare);
        case 404: return launch_sweep_t<4, 4>(L, s, prepare);
        case 408: return launch_sweep_t<4, 8>(L, s, prepare);
        case 804: return launch_sweep_t<8, 4>(L, s, prepare);
        case 808: return launch_sweep_t<8, 8>(L, s, prepare);
        case 1604: return launch_sweep_t<16, 4>(L, s, prepare);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_sweep(const SweepLaunch& L, cudaStream_t s) {
    if (L.ntiles == 0) return cudaSuccess;
    return dispatch_sweep(L, s, false);
}

cudaError_t launch_sweep_prepare(const SweepLaunch& L) {
    return dispatch_sweep(L, nullptr, true);
}

bool sweep_shape_supported(int R, int NW, int variant) {
    if (variant < 0 || variant > 6 || (variant >= 1 && variant <= 3)) return false;
    if (variant == 5 || variant == 6) {
        switch (R * 100 + NW) {
            case 402: case 404: case 408: case 804: case 808: case 1604:
                return true;
            default:
                return false;
        }
    }
    if (variant == 4) {
        switch (R * 100 + NW) {
            case 402: case 404: case 408: case 802: case 804: case 808: case 1604:
                return true;
            default:
                return false;
        }
    }
    switch (R * 100 + NW) {
        case 202: case 204: case 402: case 404: case 408: case 804: case 808: case 1604:
            return true;
        default:
            return false;
    }
}

}  // namespace logo
