// Per-thread core of the 2-opt sweep, shared by the single-instance kernel
// (sweep.cu: one CTA per tile, columns staged by TMA) and the batched kernel
// (batch.cu: whole instance in shared memory).
//
// A thread owns pair rows ib .. ib+R-1 (and row ib-1 for the reuse) and walks
// columns c upward.  With c = j + 1 (src/solvers/cpuSolver.cpp:188-230):
//     delta(i, c) = d(i, c) + d(i-1, c-1) - e[i] - e[c],  i+2 <= c <= n-1
// so each column costs R+1 distances for R pairs.  Fast path: approximate
// distances and one compare per pair against T[r] = B + e[i] + M; only
// columns where some pair passes are re-evaluated with exact_dist.
#pragma once
#include "logo_device.cuh"

namespace logo {

template <int R>
struct RowBlock {
    float x[R + 1], y[R + 1];  // rows ib-1 .. ib+R-1
    float T[R];                // filter threshold of pair row ib+r
    float Dp[R];               // approx d(ib-1+r, c-1)
};

// Loads rows ib-1 .. ib+R-1 of Q (clamped to n-1).
template <int R>
__device__ __forceinline__ void load_rows(RowBlock<R>& rb, const OrderedCity* Q,
                                          uint32_t ib, uint32_t n) {
#pragma unroll
    for (int k = 0; k <= R; ++k) {
        const uint32_t idx = min(ib - 1 + k, n - 1);
        const float4 p = *reinterpret_cast<const float4*>(Q + idx);
        rb.x[k] = p.x;
        rb.y[k] = p.y;
    }
}

template <int R>
__device__ __forceinline__ void refresh_thresholds(RowBlock<R>& rb, const OrderedCity* Q,
                                                   uint32_t ib, uint32_t n, int B,
                                                   float margin) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        if (i + 3 <= n) {
            const int ei = (int)Q[i].e;
            rb.T[r] = (float)(B + ei) + margin;
        } else {
            rb.T[r] = -INFINITY;
        }
    }
}

// Exact re-evaluation of the candidate pairs of column c.  q = column c,
// qp = column c-1.  Inlined so that the row block stays in registers.
template <int R>
__device__ __forceinline__ void column_exact(RowBlock<R>& rb, const float* Dc,
                                             const OrderedCity& q, const OrderedCity& qp,
                                             uint32_t c, uint32_t ib, uint32_t n,
                                             const OrderedCity* Q, float margin, int& B,
                                             uint64_t& best) {
    const int ec = (int)q.e;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        const float v = Dc[r + 1] + (rb.Dp[r] - q.e);
        if (c >= i + 2 && v < rb.T[r]) {
            const int d1 = exact_dist(rb.x[r + 1], rb.y[r + 1], q.x, q.y);
            const int d2 = exact_dist(rb.x[r], rb.y[r], qp.x, qp.y);
            const int ei = (int)Q[i].e;
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

// One column: cols[c - base] is column c (and cols[c - base - 1] column c-1).
template <int R, bool MASK>
__device__ __forceinline__ void column_step(RowBlock<R>& rb, const OrderedCity* cols,
                                            uint32_t base, uint32_t c, uint32_t ib,
                                            uint32_t n, const OrderedCity* Q, float margin,
                                            int& B, uint64_t& best) {
    const OrderedCity q = cols[c - base];
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
        const OrderedCity qp = cols[c - base - 1];
        column_exact<R>(rb, Dc, q, qp, c, ib, n, Q, margin, B, best);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) rb.Dp[r] = Dc[r];
}

// Walks columns [max(c_lo, ib+2), c_hi) for this thread's rows.
template <int R>
__device__ __forceinline__ void walk_columns(RowBlock<R>& rb, const OrderedCity* cols,
                                             uint32_t base, uint32_t c_lo, uint32_t c_hi,
                                             uint32_t ib, uint32_t n, const OrderedCity* Q,
                                             float margin, int& B, uint64_t& best) {
    const uint32_t c_first = max(c_lo, ib + 2);
    if (ib + 3 > n || c_first >= c_hi) return;
    const OrderedCity pc = cols[c_first - base - 1];
#pragma unroll
    for (int r = 0; r < R; ++r) rb.Dp[r] = approx_dist(rb.x[r], rb.y[r], pc.x, pc.y);
    uint32_t c = c_first;
    const uint32_t peel_end = min(c_hi, ib + R + 1);
    for (; c < peel_end; ++c)
        column_step<R, true>(rb, cols, base, c, ib, n, Q, margin, B, best);
#pragma unroll 2
    for (; c < c_hi; ++c)
        column_step<R, false>(rb, cols, base, c, ib, n, Q, margin, B, best);
}

}  // namespace logo
