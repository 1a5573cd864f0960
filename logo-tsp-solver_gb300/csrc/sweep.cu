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

namespace logo {

template <int R>
struct RowBlock {
    float x[R + 1], y[R + 1];  // rows ib-1 .. ib+R-1
    float T[R];                // filter threshold of pair row ib+r
    float Dp[R];               // approx d(ib-1+r, c-1)
};

template <int R>
__device__ __forceinline__ void refresh_thresholds(RowBlock<R>& rb,
                                                   const OrderedCity* Q,
                                                   uint32_t ib, uint32_t n,
                                                   int B, float margin) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        uint32_t i = ib + r;
        if (i + 3 <= n) {
            int ei = (int)__ldg(&Q[i].e);
            rb.T[r] = (float)(B + ei) + margin;
        } else {
            rb.T[r] = -INFINITY;
        }
    }
}

// Exact re-evaluation of the candidates of column c (rarely taken branch;
// inlined so that the row block stays in registers).
template <int R>
__device__ __forceinline__ void column_exact(RowBlock<R>& rb, const float* Dc,
                                          const OrderedCity& q,
                                          const OrderedCity& qp, uint32_t c,
                                          uint32_t ib, uint32_t n,
                                          const OrderedCity* Q, float margin,
                                          int& B, uint64_t& best) {
    const int ec = (int)q.e;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        const float v = Dc[r + 1] + (rb.Dp[r] - q.e);
        if (c >= i + 2 && v < rb.T[r]) {
            const int d1 = exact_dist(rb.x[r + 1], rb.y[r + 1], q.x, q.y);
            const int d2 = exact_dist(rb.x[r], rb.y[r], qp.x, qp.y);
            const int ei = (int)__ldg(&Q[i].e);
            const int delta = d1 + d2 - ei - ec;
            if (delta <= B) {
                const uint64_t key = pack_key(delta, i, c);
                best = key < best ? key : best;
                if (delta < B) {
                    B = delta;
                    refresh_thresholds<R>(rb, Q, ib, n, B, margin);
                }
            }
        }
    }
}

template <int R, bool MASK>
__device__ __forceinline__ void column_step(RowBlock<R>& rb,
                                            const OrderedCity* cols,
                                            uint32_t col0, uint32_t c,
                                            uint32_t ib, uint32_t n,
                                            const OrderedCity* Q, float margin,
                                            int& B, uint64_t& best) {
    const OrderedCity q = cols[c - col0 + 1];
    float Dc[R + 1];
#pragma unroll
    for (int k = 0; k <= R; ++k) Dc[k] = approx_dist(rb.x[k], rb.y[k], q.x, q.y);
    bool hit = false;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float v = Dc[r + 1] + (rb.Dp[r] - q.e);
        const bool cand = v < rb.T[r];
        if (MASK)
            hit |= cand && (c >= ib + r + 2);
        else
            hit |= cand;
    }
    if (hit) {
        const OrderedCity qp = cols[c - col0];
        column_exact<R>(rb, Dc, q, qp, c, ib, n, Q, margin, B, best);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) rb.Dp[r] = Dc[r];
}

template <int R, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_kernel(const OrderedCity* __restrict__ Q0,
                 const OrderedCity* __restrict__ Q1, uint32_t n,
                 const uint2* __restrict__ tiles, uint32_t cb, float margin,
                 DevState* st) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
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
#pragma unroll
    for (int k = 0; k <= R; ++k) {
        const uint32_t idx = min(ib - 1 + k, n - 1);
        const float4 p = __ldg(reinterpret_cast<const float4*>(Q + idx));
        rb.x[k] = p.x;
        rb.y[k] = p.y;
    }
    refresh_thresholds<R>(rb, Q, ib, n, B, margin);

    const bool staged = mbar_wait_bounded(bar, 0, &st->status);
    const uint32_t c_first = max(col0, ib + 2);
    if (staged && ib + 3 <= n && c_first < col_end) {
        const OrderedCity pc = cols[c_first - col0];
#pragma unroll
        for (int r = 0; r < R; ++r) rb.Dp[r] = approx_dist(rb.x[r], rb.y[r], pc.x, pc.y);
        uint32_t c = c_first;
        const uint32_t peel_end = min(col_end, ib + R + 1);
        for (; c < peel_end; ++c)
            column_step<R, true>(rb, cols, col0, c, ib, n, Q, margin, B, best);
#pragma unroll 2
        for (; c < col_end; ++c)
            column_step<R, false>(rb, cols, col0, c, ib, n, Q, margin, B, best);
    }

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

template <int R, int NW>
static cudaError_t launch_sweep_t(const SweepLaunch& L, cudaStream_t s, bool prepare) {
    const size_t smem = sweep_smem_bytes(L.cb);
    if (prepare) {
        // opt-in above 48 KB; called once per shape, outside stream capture
        return cudaFuncSetAttribute(sweep_kernel<R, NW>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(smem > 48 * 1024 ? smem : 48 * 1024));
    }
    sweep_kernel<R, NW><<<L.ntiles, NW * 32, smem, s>>>(L.Q0, L.Q1, L.n, L.tiles,
                                                        L.cb, L.margin, L.st);
    return cudaGetLastError();
}

static cudaError_t dispatch_sweep(const SweepLaunch& L, cudaStream_t s, bool prepare) {
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

bool sweep_shape_supported(int R, int NW) {
    switch (R * 100 + NW) {
        case 202: case 204: case 402: case 404: case 408: case 804: case 808: case 1604:
            return true;
        default:
            return false;
    }
}

}  // namespace logo
