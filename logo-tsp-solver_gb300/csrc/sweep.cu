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
#include "logo_device.cuh"
#include "logo_internal.h"
#include "sweep_core.cuh"
#include "sweep_core2.cuh"
#include "sweep_core3.cuh"
#include "sweep_core4.cuh"
#include "sweep_core5.cuh"
#include "sweep_core6.cuh"

namespace logo {

template <int R, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel(const OrderedCity* __restrict__ Q0,
                 const OrderedCity* __restrict__ Q1, uint32_t n,
                 const uint2* __restrict__ tiles, uint32_t cb, float margin,
                 DevState* st) {
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

// Square-root-free variant (sweep_core3.cuh): same tiling and staging as
// sweep_kernel; the fast path needs no MUFU operation.
template <int R, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel3(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                  uint32_t n, const uint2* __restrict__ tiles, uint32_t cb, DevState* st) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* wbest = reinterpret_cast<uint64_t*>(smem_raw + 8);  // NW <= 8
    OrderedCity* cols = reinterpret_cast<OrderedCity*>(smem_raw + 80);

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
    RowBlock3<R> rb;
    load_rows3<R>(rb, Q, ib, n);
    refresh_thresholds3<R>(rb, Q, ib, n, B);
    if (mbar_wait_bounded(bar, 0, &st->status))
        walk_columns3<R>(rb, cols, col0 - 1, col0, col_end, ib, n, Q, B, best);

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

// Packed square-root-free variant (sweep_core4.cuh): the staged tile is
// re-laid out as broadcast records plus the largest edge of every 32-column
// window.
__host__ __device__ constexpr size_t sweep4_cols_offset(uint32_t cb) {
    return (96 + (size_t)(cb + 1) * sizeof(OrderedCity) + 31) & ~(size_t)31;
}
__host__ __device__ constexpr size_t sweep4_wmax_offset(uint32_t cb) {
    return sweep4_cols_offset(cb) + (size_t)(cb + 1) * sizeof(ColRec);
}

template <int R, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel4(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                  uint32_t n, const uint2* __restrict__ tiles, uint32_t cb, DevState* st) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* wbest = reinterpret_cast<uint64_t*>(smem_raw + 8);  // NW <= 8
    OrderedCity* stage = reinterpret_cast<OrderedCity*>(smem_raw + 96);
    ColRec* cols = reinterpret_cast<ColRec*>(smem_raw + sweep4_cols_offset(cb));
    float* wmax = reinterpret_cast<float*>(smem_raw + sweep4_wmax_offset(cb));

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
    uint64_t best = kNoMove;
    int B = -1;
    {
        const uint64_t gk = *(volatile unsigned long long*)&st->best_key;
        if (gk != kNoMove) B = min(B, key_delta(gk));
    }
    RowBlock4<R> rb;
    load_rows4<R>(rb, Q, ib, n);
    refresh4<R>(rb, Q, ib, n, B);
    const bool staged = mbar_wait_bounded(bar, 0, &st->status);
    const uint32_t nwin = (col_end - col0 + kWin - 1) / kWin;
    if (staged) {
        for (uint32_t k = threadIdx.x; k < ncols; k += NW * 32) cols[k] = make_colrec(stage[k]);
        for (uint32_t w = threadIdx.x; w < nwin; w += NW * 32) {
            const uint32_t a = 1 + w * kWin, b = min(a + kWin, ncols);
            float m = 0.f;
            for (uint32_t k = a; k < b; ++k) m = fmaxf(m, stage[k].e);
            wmax[w] = m;
        }
    }
    __syncthreads();
    if (staged)
        walk_columns4<R>(rb, cols, col0 - 1, wmax, col0, col0, col_end, ib, n, Q, B, best);

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

__host__ __device__ constexpr size_t sweep5_hot_offset(uint32_t cb) {
    return 96 + (size_t)(cb + 1) * sizeof(OrderedCity);
}
__host__ __device__ constexpr size_t sweep5_wmax_offset(uint32_t cb) {
    return sweep5_hot_offset(cb) + (size_t)(cb + 1) * sizeof(float4);
}

template <int R, int NW, int G>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel5(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                  uint32_t n, const uint2* __restrict__ tiles, uint32_t cb, DevState* st) {
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
                  uint32_t n, const uint2* __restrict__ tiles, uint32_t cb, DevState* st) {
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
        walk_columns6<R, G>(rb, t, wmax, col0, col0, col_end, ib, n, st, bs);
    }

    const uint64_t best = warp_min_u64(bs.best);
    if (lane == 0 && best != kNoMove) atomicMin(&st->best_key, (unsigned long long)best);
}

__host__ __device__ constexpr size_t sweep2_cols_offset(uint32_t cb) {
    return (96 + (size_t)(cb + 1) * sizeof(OrderedCity) + 31) & ~(size_t)31;
}

// Packed variant: the staged tile is re-laid out in shared memory as 32-byte
// broadcast records (sweep_core2.cuh) so the fast path issues f32x2 FFMA2 /
// FMUL2 / FADD2 for two rows at a time.
template <int R, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel2(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                  uint32_t n, const uint2* __restrict__ tiles, uint32_t cb, float margin,
                  DevState* st) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* wbest = reinterpret_cast<uint64_t*>(smem_raw + 8);  // NW <= 8
    OrderedCity* stage = reinterpret_cast<OrderedCity*>(smem_raw + 96);
    ColRec* cols = reinterpret_cast<ColRec*>(smem_raw + sweep2_cols_offset(cb));

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
    uint64_t best = kNoMove;
    int B = -1;
    {
        const uint64_t gk = *(volatile unsigned long long*)&st->best_key;
        if (gk != kNoMove) B = min(B, key_delta(gk));
    }
    RowBlock2<R> rb;
    load_rows2<R>(rb, Q, ib, n);
    refresh_thresholds2<R>(rb, Q, ib, n, B, margin);
    const bool staged = mbar_wait_bounded(bar, 0, &st->status);
    if (staged)
        for (uint32_t k = threadIdx.x; k < ncols; k += NW * 32) cols[k] = make_colrec(stage[k]);
    __syncthreads();
    if (staged)
        walk_columns2<R>(rb, cols, col0 - 1, col0, col_end, ib, n, Q, margin, B, best);

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

size_t sweep_smem_bytes(uint32_t cb) { return 80 + (size_t)(cb + 1) * sizeof(OrderedCity); }
size_t sweep2_smem_bytes(uint32_t cb) {
    return sweep2_cols_offset(cb) + (size_t)(cb + 1) * sizeof(ColRec);
}

// The dynamic shared-memory limit is a property of the kernel, shared by
// every context in the process: it is always set for the largest tile a
// context may choose (4096 columns), never for this context's own tile, so
// that contexts created later cannot lower it under another one's launch.
constexpr uint32_t kMaxTileCols = 4096;
inline int attr_bytes(size_t smem) { return (int)(smem > 48 * 1024 ? smem : 48 * 1024); }

template <int R, int NW>
static cudaError_t launch_sweep2_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = sweep2_smem_bytes(L.cb);
    if (prepare) {
        return cudaFuncSetAttribute(sweep_kernel2<R, NW>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    attr_bytes(sweep2_smem_bytes(kMaxTileCols)));
    }
    sweep_kernel2<R, NW><<<L.ntiles, NW * 32, smem, s>>>(L.Q0, L.Q1, L.n, L.tiles, L.cb,
                                                         L.margin, L.st);
    return cudaGetLastError();
}

size_t sweep4_smem_bytes(uint32_t cb) {
    return sweep4_wmax_offset(cb) + ((size_t)cb / kWin + 2) * sizeof(float);
}

template <int R, int NW>
static cudaError_t launch_sweep4_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = sweep4_smem_bytes(L.cb);
    if (prepare) {
        return cudaFuncSetAttribute(sweep_kernel4<R, NW>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    attr_bytes(sweep4_smem_bytes(kMaxTileCols)));
    }
    sweep_kernel4<R, NW><<<L.ntiles, NW * 32, smem, s>>>(L.Q0, L.Q1, L.n, L.tiles, L.cb, L.st);
    return cudaGetLastError();
}

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
    sweep_kernel5<R, NW, G><<<L.ntiles, NW * 32, smem, s>>>(L.Q0, L.Q1, L.n, L.tiles, L.cb,
                                                           L.st);
    return cudaGetLastError();
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
    sweep_kernel6<R, NW, G><<<L.ntiles, NW * 32, smem, s>>>(L.Q0, L.Q1, L.n, L.tiles, L.cb,
                                                           L.st);
    return cudaGetLastError();
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
static cudaError_t launch_sweep3_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = sweep_smem_bytes(L.cb);
    if (prepare) {
        return cudaFuncSetAttribute(sweep_kernel3<R, NW>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    attr_bytes(sweep_smem_bytes(kMaxTileCols)));
    }
    sweep_kernel3<R, NW><<<L.ntiles, NW * 32, smem, s>>>(L.Q0, L.Q1, L.n, L.tiles, L.cb, L.st);
    return cudaGetLastError();
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
    sweep_kernel<R, NW><<<L.ntiles, NW * 32, smem, s>>>(L.Q0, L.Q1, L.n, L.tiles,
                                                        L.cb, L.margin, L.st);
    return cudaGetLastError();
}

static cudaError_t dispatch_sweep(const SweepLaunch& L, cudaStream_t s, bool prepare) {
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
    if (L.variant == 3) {
        switch (L.R * 100 + L.NW) {
            case 404: return launch_sweep4_t<4, 4>(L, s, prepare);
            case 804: return launch_sweep4_t<8, 4>(L, s, prepare);
            case 808: return launch_sweep4_t<8, 8>(L, s, prepare);
            case 1604: return launch_sweep4_t<16, 4>(L, s, prepare);
            default: return cudaErrorInvalidValue;
        }
    }
    if (L.variant == 2) {
        switch (L.R * 100 + L.NW) {
            case 202: return launch_sweep3_t<2, 2>(L, s, prepare);
            case 402: return launch_sweep3_t<4, 2>(L, s, prepare);
            case 404: return launch_sweep3_t<4, 4>(L, s, prepare);
            case 804: return launch_sweep3_t<8, 4>(L, s, prepare);
            case 808: return launch_sweep3_t<8, 8>(L, s, prepare);
            case 1604: return launch_sweep3_t<16, 4>(L, s, prepare);
            default: return cudaErrorInvalidValue;
        }
    }
    if (L.variant == 1) {
        switch (L.R * 100 + L.NW) {
            case 402: return launch_sweep2_t<4, 2>(L, s, prepare);
            case 404: return launch_sweep2_t<4, 4>(L, s, prepare);
            case 804: return launch_sweep2_t<8, 4>(L, s, prepare);
            case 808: return launch_sweep2_t<8, 8>(L, s, prepare);
            case 1602: return launch_sweep2_t<16, 2>(L, s, prepare);
            case 1604: return launch_sweep2_t<16, 4>(L, s, prepare);
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
    if (variant == 5) {
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
    if (variant == 3) {
        switch (R * 100 + NW) {
            case 404: case 804: case 808: case 1604:
                return true;
            default:
                return false;
        }
    }
    if (variant == 2) {
        switch (R * 100 + NW) {
            case 202: case 402: case 404: case 804: case 808: case 1604:
                return true;
            default:
                return false;
        }
    }
    if (variant == 1) {
        switch (R * 100 + NW) {
            case 402: case 404: case 804: case 808: case 1602: case 1604:
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
