// CTA-level tour operations on one instance held by one CTA (in shared or
// global memory): the in-place move / kick permutations, edge and length
// recomputation and a full best-improvement sweep.  Used by the batched
// persistent solver (batch.cu) and the serving rounds (serve.cu).
//
//   rotate_reverse  ≙ rotate + reverse, src/solvers/twoOptLocalSolver.cpp:41-48
//                     and ILSGlobalSolver::kick, src/solvers/ILSGlobalSolver.cpp:37-48,
//                     done in place as rev[p,q) || rev[q,n), then rev[0,q)
//   double_bridge   old[0,p1) old[p2,p3) old[p1,p2) old[p3,n) as
//                     rev[p1,p3), then rev[p1,m) || rev[m,p3)
//   tour_length     ≙ routeLength, src/headers.h:170-189
//   sweep           ≙ the CPUSolver::optimizeStep loop (src/solvers/cpuSolver.cpp:188-230)
//                     over warp tiles of 32R rows x TC columns
//   sweep_boxed     the same, skipping the 32-column windows that the box
//                     test of sweep_core7.cuh closes for a lane's rows
#pragma once
#include <cstdint>

#include "logo_device.cuh"
#include "sweep_core.cuh"
#include "sweep_core7.cuh"

namespace logo {

template <int NT>
struct CtaShared {
    unsigned long long wbest[NT / 32];
    unsigned long long wsum[NT / 32];
    unsigned long long key;
    unsigned long long sum;
    unsigned int idx;
    unsigned int p, q, r;  // permutation parameters broadcast by thread 0
    unsigned int tiles_before[72];
};

__device__ __forceinline__ void swap_q(OrderedCity* Q, uint32_t* route, uint32_t a,
                                       uint32_t b) {
    const float4 qa = *reinterpret_cast<float4*>(Q + a);
    const float4 qb = *reinterpret_cast<float4*>(Q + b);
    *reinterpret_cast<float4*>(Q + a) = qb;
    *reinterpret_cast<float4*>(Q + b) = qa;
    const uint32_t ra = route[a];
    route[a] = route[b];
    route[b] = ra;
}

// Reverses [a0, a1) and [b0, b1) (disjoint) in one pass.
template <int NT>
__device__ __forceinline__ void reverse2(OrderedCity* Q, uint32_t* route, uint32_t a0,
                                         uint32_t a1, uint32_t b0, uint32_t b1) {
    const uint32_t ha = (a1 - a0) / 2, hb = (b1 - b0) / 2;
    for (uint32_t t = threadIdx.x; t < ha + hb; t += NT) {
        if (t < ha)
            swap_q(Q, route, a0 + t, a1 - 1 - t);
        else
            swap_q(Q, route, b0 + (t - ha), b1 - 1 - (t - ha));
    }
}

template <int NT>
__device__ __forceinline__ void recompute_edges(OrderedCity* Q, uint32_t n) {
    for (uint32_t k = threadIdx.x; k < n; k += NT) {
        const OrderedCity a = Q[k];
        const OrderedCity b = Q[k == 0 ? n - 1 : k - 1];
        Q[k].e = (float)exact_dist(b.x, b.y, a.x, a.y);
    }
}

// new = old[p..q) ++ rev(old[0..p)) ++ rev(old[q..n)), p <= q.
template <int NT>
__device__ __forceinline__ void rotate_reverse(OrderedCity* Q, uint32_t* route, uint32_t n,
                                               uint32_t p, uint32_t q) {
    reverse2<NT>(Q, route, p, q, q, n);
    __syncthreads();
    reverse2<NT>(Q, route, 0, q, 0, 0);
    __syncthreads();
    recompute_edges<NT>(Q, n);
    __syncthreads();
}

// new = old[0,p1) old[p2,p3) old[p1,p2) old[p3,n).
template <int NT>
__device__ __forceinline__ void double_bridge(OrderedCity* Q, uint32_t* route, uint32_t n,
                                              uint32_t p1, uint32_t p2, uint32_t p3) {
    reverse2<NT>(Q, route, p1, p3, 0, 0);
    __syncthreads();
    const uint32_t m = p1 + (p3 - p2);
    reverse2<NT>(Q, route, p1, m, m, p3);
    __syncthreads();
    recompute_edges<NT>(Q, n);
    __syncthreads();
}

template <int NT>
__device__ __forceinline__ unsigned long long block_sum(CtaShared<NT>& S,
                                                        unsigned long long v) {
    v = warp_sum_u64(v);
    if ((threadIdx.x & 31) == 0) S.wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; ++w) t += S.wsum[w];
        S.sum = t;
    }
    __syncthreads();
    const unsigned long long r = S.sum;
    __syncthreads();
    return r;
}

template <int NT>
__device__ __forceinline__ unsigned long long tour_length(CtaShared<NT>& S,
                                                          const OrderedCity* Q, uint32_t n) {
    unsigned long long s = 0;
    for (uint32_t k = threadIdx.x; k < n; k += NT) s += (unsigned long long)Q[k].e;
    return block_sum<NT>(S, s);
}

// One best-improvement sweep of the resident instance; returns the packed
// key of the best move (kNoMove if none).  Work: warp tiles of 32R rows x TC
// columns dealt round-robin to the warps.
template <int R, int NT, int TC>
__device__ __forceinline__ unsigned long long sweep(CtaShared<NT>& S, const OrderedCity* Q,
                                                    uint32_t n, float margin) {
    constexpr int NW = NT / 32;
    constexpr uint32_t RT = 32 * R;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t best = kNoMove;
    if (n >= 4) {
        const uint32_t nrb = (n - 3 + RT - 1) / RT;  // row blocks over rows 1..n-3
        const uint32_t total = S.tiles_before[nrb];
        uint32_t rbk = 0;
        for (uint32_t t = warp; t < total; t += NW) {
            while (S.tiles_before[rbk + 1] <= t) ++rbk;
            const uint32_t row0 = 1 + rbk * RT;
            const uint32_t col0 = row0 + 2 + (t - S.tiles_before[rbk]) * TC;
            const uint32_t col1 = min(col0 + TC, n);
            const uint32_t ib = row0 + lane * R;
            int B = -1;
            RowBlock<R> rb;
            load_rows<R>(rb, Q, ib, n);
            refresh_thresholds<R>(rb, Q, ib, n, B, margin);
            walk_columns<R>(rb, Q, 0, col0, col1, ib, n, Q, margin, B, best);
        }
    }
    best = warp_min_u64(best);
    if (lane == 0) S.wbest[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = S.wbest[0];
#pragma unroll
        for (int w = 1; w < NW; ++w) m = S.wbest[w] < m ? S.wbest[w] : m;
        S.key = m;
    }
    __syncthreads();
    const unsigned long long k = S.key;
    __syncthreads();
    return k;
}


// Bounding box and largest edge of every window of 32 columns (columns
// 3 + 32 g .. 3 + 32 g + 31, below n) of the resident tour, for
// sweep_boxed; up to kCtaWindows windows (tours up to 4096 cities).
constexpr uint32_t kCtaWindows = 130;
struct CtaWindows {
    float4 box[kCtaWindows];  // (x0, x1, y0, y1)
    float emax[kCtaWindows];
};

template <int NT>
__device__ __forceinline__ void window_stats_cta(CtaWindows& W, const OrderedCity* Q,
                                                 uint32_t n) {
    const uint32_t nwin = n < 4 ? 0u : (n - 3 + kWin7 - 1) / kWin7;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t g = threadIdx.x >> 5; g < nwin; g += NT / 32) {  // whole warps
        const uint32_t c = 3 + g * kWin7 + lane;
        const bool in = c < n;
        const OrderedCity q = Q[in ? c : n - 1];
        float m = in ? q.e : 0.f;
        float x0 = in ? q.x : FLT_MAX, x1 = in ? q.x : -FLT_MAX;
        float y0 = in ? q.y : FLT_MAX, y1 = in ? q.y : -FLT_MAX;
        for (int o = 16; o; o >>= 1) {
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
            x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
            y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
            y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        }
        if (lane == 0) {
            W.box[g] = make_float4(x0, x1, y0, y1);
            W.emax[g] = m;
        }
    }
}

// sweep() with the window test: each lane walks a window of its tile only
// when the bounding box of its rows and the window's box let some pair be
// chosen with its current B (box_gap_pass, u = B + max e[i] + 5 + the
// window's largest edge, which bounds every V + 5 of those pairs).  W must
// hold the current tour's windows (window_stats_cta, then a barrier).  Tile
// columns start at 3 + 32k (32R-row blocks, TC a multiple of 32), so every
// window lies in one tile.
template <int R, int NT, int TC>
__device__ __forceinline__ unsigned long long sweep_boxed(CtaShared<NT>& S, const CtaWindows& W,
                                                          const OrderedCity* Q, uint32_t n,
                                                          float margin) {
    static_assert(TC % kWin7 == 0, "tile columns start at 3 + 32k");
    constexpr int NW = NT / 32;
    constexpr uint32_t RT = 32 * R;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t best = kNoMove;
    if (n >= 4) {
        const uint32_t nrb = (n - 3 + RT - 1) / RT;  // row blocks over rows 1..n-3
        const uint32_t total = S.tiles_before[nrb];
        uint32_t rbk = 0;
        for (uint32_t t = warp; t < total; t += NW) {
            while (S.tiles_before[rbk + 1] <= t) ++rbk;
            const uint32_t row0 = 1 + rbk * RT;
            const uint32_t col0 = row0 + 2 + (t - S.tiles_before[rbk]) * TC;
            const uint32_t col1 = min(col0 + TC, n);
            const uint32_t ib = row0 + lane * R;
            if (ib + 3 > n) continue;  // no pairs in this lane's rows
            int B = -1;
            RowBlock<R> rb;
            load_rows<R>(rb, Q, ib, n);
            refresh_thresholds<R>(rb, Q, ib, n, B, margin);
            float emax_rows = -3.0e7f;
            float4 box = make_float4(rb.x[1], rb.x[1], rb.y[1], rb.y[1]);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (ib + r + 3 <= n) emax_rows = fmaxf(emax_rows, Q[ib + r].e);
                box.x = fminf(box.x, rb.x[r + 1]);
                box.y = fmaxf(box.y, rb.x[r + 1]);
                box.z = fminf(box.z, rb.y[r + 1]);
                box.w = fmaxf(box.w, rb.y[r + 1]);
            }
            for (uint32_t c = col0; c < col1;) {
                const uint32_t g = (c - 3) / kWin7;
                const uint32_t wend = min(3 + (g + 1) * kWin7, col1);
                if (wend > ib + 2 &&
                    box_gap_pass(box, W.box[g], ((float)(B + 5) + emax_rows) + W.emax[g]))
                    walk_columns<R>(rb, Q, 0, c, wend, ib, n, Q, margin, B, best);
                c = wend;
            }
        }
    }
    best = warp_min_u64(best);
    if (lane == 0) S.wbest[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = S.wbest[0];
#pragma unroll
        for (int w = 1; w < NW; ++w) m = S.wbest[w] < m ? S.wbest[w] : m;
        S.key = m;
    }
    __syncthreads();
    const unsigned long long k = S.key;
    __syncthreads();
    return k;
}

// Tiles per row block of the pair triangle (rows 1..n-3) for sweep(); one
// thread of the CTA fills the table, callers synchronise afterwards.
template <int R, int TC, typename SharedT>
__device__ __forceinline__ void fill_tile_table(SharedT& S, uint32_t n) {
    constexpr uint32_t RT = 32 * R;
    uint32_t acc = 0, rbk = 0;
    S.tiles_before[0] = 0;
    if (n >= 4) {
        for (uint32_t row0 = 1; row0 + 3 <= n; row0 += RT, ++rbk) {
            acc += (n - row0 - 2 + TC - 1) / TC;
            S.tiles_before[rbk + 1] = acc;
        }
    }
}

}  // namespace logo
