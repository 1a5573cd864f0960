// Boxed screen of the sweep (LOGO_SWEEP_BOXED).
//
// Pairs are decided in blocks before any per-pair work.  For a block of rows
// (one row, or the R rows of a thread) with bounding box A and a window of
// 32 columns with bounding box W (both over the global binary32
// coordinates), and u >= V + 5 for every pair of the block (V = B + e[i] +
// e[c], B <= -1 the best exact delta known), the block can only hold a
// chosen pair if
//     s < RN(u^2),  s = RN(gy^2 + RN(gx^2)),
// gx, gy the gaps between A and W per axis (0 where they overlap).
//
// Why no chosen pair is missed.  For a row i in A and a column c in W,
// |x_i - x_c| >= gx where gx is the real gap, and the gap is one exact
// binary32 difference (W.x0 - A.x1 or A.x0 - W.x1), so rounding is
// monotone: |RN(x_i - x_c)| >= RN(gx).  The reference squares
// dx = RN(x_i - x_c), dy = RN(y_i - y_c); two roundings, each up by at most
// 2^-24 relative, give dx^2 + dy^2 >= s (1 + 2^-24)^-2.  A chosen pair needs
// dx^2 + dy^2 < (V + 0.5)^2 (1 + 2^-22) (sweep_core5.cuh), so
// s < (V + 0.5)^2 (1 + 2^-21) <= (V + 5)^2 (1 - 2^-24) <= RN(u^2) for every
// V < 1.6e7 (here V < 4e6).  Rows without pairs get u = -3e7 and never pass.
//
// Blocks that pass become units (a thread's rows that passed their own
// one-row test, times one window); a warp evaluates a unit with one lane per
// column: the squared screen of sweep_core3.cuh on the pair (max of the two
// sums of squares against RN(u |u|), u = B + e[i] + 5 + e[c]) and the exact
// distances where it passes.  Lowering B only tightens every test.
#pragma once
#include <cfloat>
#include "sweep_core3.cuh"
#include "sweep_core5.cuh"

namespace logo {

constexpr uint32_t kWin7 = 32;

// The block test above for boxes a, b given as (x0, x1, y0, y1).
__device__ __forceinline__ bool box_gap_pass(float4 a, float4 b, float u) {
    const float gx = fmaxf(fmaxf(__fsub_rn(b.x, a.y), __fsub_rn(a.x, b.y)), 0.f);
    const float gy = fmaxf(fmaxf(__fsub_rn(b.z, a.w), __fsub_rn(a.z, b.w)), 0.f);
    const float s = __fmaf_rn(gy, gy, __fmul_rn(gx, gx));
    return u > 0.f && s < __fmul_rn(u, u);
}

template <int R>
struct RowBlock7 {
    float x[R], y[R];  // rows ib .. ib + R - 1
    float T2[R];       // B + e[ib + r] + 5, or -3e7 for rows without pairs
    float4 box;        // bounding box of the R rows
    float T2max;       // max over r of T2[r]
};

template <int R>
__device__ __forceinline__ void load_rows7(RowBlock7<R>& rb, const OrderedCity* Q, uint32_t ib,
                                           uint32_t n, int B) {
    rb.T2max = -3.0e7f;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        const OrderedCity z = Q[min(i, n - 1)];
        rb.x[r] = z.x;
        rb.y[r] = z.y;
        rb.T2[r] = (i + 3 <= n) ? (float)(B + (int)z.e + 5) : -3.0e7f;
        rb.T2max = fmaxf(rb.T2max, rb.T2[r]);
    }
    rb.box = make_float4(rb.x[0], rb.x[0], rb.y[0], rb.y[0]);
#pragma unroll
    for (int r = 1; r < R; ++r) {
        rb.box.x = fminf(rb.box.x, rb.x[r]);
        rb.box.y = fmaxf(rb.box.y, rb.x[r]);
        rb.box.z = fminf(rb.box.z, rb.y[r]);
        rb.box.w = fmaxf(rb.box.w, rb.y[r]);
    }
}

// Rows of the block that may hold a chosen pair in the window (box w,
// largest edge E): the block test first, then one test per row.
template <int R>
__device__ __forceinline__ uint32_t rows_open7(const RowBlock7<R>& rb, float4 w, float E) {
    if (!box_gap_pass(rb.box, w, rb.T2max + E)) return 0u;
    uint32_t rm = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float4 p = make_float4(rb.x[r], rb.x[r], rb.y[r], rb.y[r]);
        rm |= (uint32_t)box_gap_pass(p, w, rb.T2[r] + E) << r;
    }
    return rm;
}

// One unit: rows uib + r (bit r of rm) against column c (this lane's
// column of the window; c < col_end).  stg[k] = column col0 - 1 + k.  The
// unit's rows are read from global memory (L2) all at once for R <= 8, so a
// unit waits for one round trip rather than one per open row (heavy tiles
// queue tens of units per warp).
template <int R>
__device__ __forceinline__ void unit_pair7(const OrderedCity& a, const OrderedCity& ap,
                                           const OrderedCity& q, const OrderedCity& qp,
                                           uint32_t i, uint32_t c, float M, int& B,
                                           uint64_t& best) {
    const int ei = (int)a.e, ec = (int)q.e;
    const float u = (float)(B + ei + 5) + q.e;
    const float L = u * fabsf(u);
    if (fmaxf(sq_dist(a.x, a.y, q.x, q.y), sq_dist(ap.x, ap.y, qp.x, qp.y)) < L &&
        approx_delta_pass(a.x, a.y, ap.x, ap.y, q, qp, ei, B, M)) {
        const int d1 = exact_dist(a.x, a.y, q.x, q.y);
        const int d2 = exact_dist(ap.x, ap.y, qp.x, qp.y);
        const int delta = d1 + d2 - ei - ec;
        if (delta <= B) {
            const uint64_t key = pack_key(delta, i, c);
            best = key < best ? key : best;
            B = delta < B ? delta : B;
        }
    }
}

template <int R>
__device__ __forceinline__ void unit7(const OrderedCity* Q, const OrderedCity* stg,
                                      uint32_t col0, uint32_t c, uint32_t uib, uint32_t rm,
                                      uint32_t n, float M, int& B, uint64_t& best) {
    const uint32_t k = c - col0 + 1;
    const OrderedCity q = stg[k], qp = stg[k - 1];
    if constexpr (R <= 8) {
        OrderedCity rw[R + 1];  // rows uib - 1 .. uib + R - 1 (uib >= 1)
#pragma unroll
        for (int t = 0; t <= R; ++t) rw[t] = Q[min(uib - 1 + t, n - 1)];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t i = uib + r;
            if (!((rm >> r) & 1u) || c < i + 2 || i + 3 > n) continue;
            unit_pair7<R>(rw[r + 1], rw[r], q, qp, i, c, M, B, best);
        }
    } else {
#pragma unroll 1
        for (uint32_t m = rm; m; m &= m - 1) {
            const uint32_t i = uib + (__ffs(m) - 1);
            if (c < i + 2 || i + 3 > n) continue;
            unit_pair7<R>(Q[i], Q[i - 1], q, qp, i, c, M, B, best);
        }
    }
}

}  // namespace logo
