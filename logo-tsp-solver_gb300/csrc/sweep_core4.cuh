// Square-root-free sweep core with packed f32x2 distances and windowed row
// thresholds (LOGO_SWEEP_SQUARED_PACKED).
//
// The screen of sweep_core3.cuh needs, per pair, u = B + e[i] + 5 + e[c] and
// L = u*|u|.  Here the column term is bounded over a window of kWin columns:
// with E = max e[c] over the window, L_row = (B + e[i] + 5 + E) * |...| is at
// least every pair's own L in that window (u*|u| grows with u), so
//     max(s(i,c), s(i-1,c-1)) < L_row
// is a superset test computed once per row per window.  Per pair the fast
// path is then one FMNMX and one FSETP; the sums of squares of two rows at a
// time are FFMA2/FMUL2/FFMA2 on register pairs.  A column where some pair
// passes is re-checked with the exact per-pair L and evaluated exactly, as in
// sweep_core3.cuh, so the chosen move is unchanged.
#pragma once
#include "sweep_core2.cuh"
#include "sweep_core3.cuh"

namespace logo {

constexpr uint32_t kWin = 32;

// R even; rows ib-1 .. ib+R-1 as packs (2m, 2m+1), m < R/2, plus row R.
template <int R>
struct RowBlock4 {
    float2 x[R / 2], y[R / 2];
    float xs, ys;
    float T2[R];     // B + e[ib+r] + 5
    float L[R];      // window threshold of pair row r
    float2 Sp[R / 2];  // s(row k, c-1) for k = 0..R-1
};

template <int R>
__device__ __forceinline__ void load_rows4(RowBlock4<R>& rb, const OrderedCity* Q, uint32_t ib,
                                           uint32_t n) {
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const OrderedCity a = Q[min(ib - 1 + 2 * m, n - 1)], b = Q[min(ib + 2 * m, n - 1)];
        rb.x[m] = make_float2(a.x, b.x);
        rb.y[m] = make_float2(a.y, b.y);
    }
    const OrderedCity z = Q[min(ib - 1 + R, n - 1)];
    rb.xs = z.x;
    rb.ys = z.y;
}

template <int R>
__device__ __forceinline__ void refresh4(RowBlock4<R>& rb, const OrderedCity* Q, uint32_t ib,
                                         uint32_t n, int B) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        rb.T2[r] = (i + 3 <= n) ? (float)(B + (int)Q[i].e + 5) : -3.0e7f;
    }
}

template <int R>
__device__ __forceinline__ void window_thresholds(RowBlock4<R>& rb, float emax) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float u = rb.T2[r] + emax;
        rb.L[r] = u * fabsf(u);
    }
}

template <int R>
__device__ __forceinline__ float row_x4(const RowBlock4<R>& rb, int k) {
    return k == R ? rb.xs : ((k & 1) ? rb.x[k >> 1].y : rb.x[k >> 1].x);
}
template <int R>
__device__ __forceinline__ float row_y4(const RowBlock4<R>& rb, int k) {
    return k == R ? rb.ys : ((k & 1) ? rb.y[k >> 1].y : rb.y[k >> 1].x);
}

template <int R>
__device__ __forceinline__ void sq_packed(const RowBlock4<R>& rb, const ColRec& q, float2* S,
                                          float& Ss) {
    const float2 neg1 = make_float2(-1.f, -1.f);
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const float2 dx = __ffma2_rn(q.x, neg1, rb.x[m]);
        const float2 dy = __ffma2_rn(q.y, neg1, rb.y[m]);
        S[m] = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
    }
    Ss = sq_dist(rb.xs, rb.ys, q.x.x, q.y.x);
}

// Exact per-pair re-check and evaluation of column c (q = column c,
// qp = column c-1).  S: packs of s(row k, c), Ss: s(row R, c).
template <int R>
__device__ __forceinline__ void column_exact4(RowBlock4<R>& rb, const float2* S, float Ss,
                                              const ColRec& q, const ColRec& qp, uint32_t c,
                                              uint32_t ib, uint32_t n, const OrderedCity* Q,
                                              float emax, int& B, uint64_t& best) {
    const int ec = (int)q.e.x;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        const float scur = (r + 1 == R) ? Ss : pair_of(S, r + 1);
        const float sprev = pair_of(rb.Sp, r);
        const float u = rb.T2[r] + q.e.x;
        const float L = u * fabsf(u);
        if (c >= i + 2 && fmaxf(scur, sprev) < L) {
            const int d1 = exact_dist(row_x4<R>(rb, r + 1), row_y4<R>(rb, r + 1), q.xy.x, q.xy.y);
            const int d2 = exact_dist(row_x4<R>(rb, r), row_y4<R>(rb, r), qp.xy.x, qp.xy.y);
            const int ei = (int)Q[i].e;
            const int delta = d1 + d2 - ei - ec;
            if (delta <= B) {
                const uint64_t key = pack_key(delta, i, c);
                best = key < best ? key : best;
                if (delta < B) {
                    B = delta;
                    refresh4<R>(rb, Q, ib, n, B);
                    window_thresholds<R>(rb, emax);
                }
            }
        }
    }
}

template <int R, bool MASK>
__device__ __forceinline__ void column_step4(RowBlock4<R>& rb, const ColRec* cols, uint32_t base,
                                             uint32_t c, uint32_t ib, uint32_t n,
                                             const OrderedCity* Q, float emax, int& B,
                                             uint64_t& best) {
    const ColRec q = cols[c - base];
    float2 S[R / 2];
    float Ss;
    sq_packed<R>(rb, q, S, Ss);
    bool hit = false;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float scur = (r + 1 == R) ? Ss : pair_of(S, r + 1);
        const bool cand = fmaxf(scur, pair_of(rb.Sp, r)) < rb.L[r];
        if (MASK)
            hit |= cand && (c >= ib + r + 2);
        else
            hit |= cand;
    }
    if (hit) {
        const ColRec qp = cols[c - base - 1];
        column_exact4<R>(rb, S, Ss, q, qp, c, ib, n, Q, emax, B, best);
    }
#pragma unroll
    for (int m = 0; m < R / 2; ++m) rb.Sp[m] = S[m];
}

// cols[c - base] is column c; wmax[w] the largest e over columns
// [wbase + w*kWin, wbase + (w+1)*kWin).
template <int R>
__device__ __forceinline__ void walk_columns4(RowBlock4<R>& rb, const ColRec* cols, uint32_t base,
                                              const float* wmax, uint32_t wbase, uint32_t c_lo,
                                              uint32_t c_hi, uint32_t ib, uint32_t n,
                                              const OrderedCity* Q, int& B, uint64_t& best) {
    const uint32_t c_first = max(c_lo, ib + 2);
    if (ib + 3 > n || c_first >= c_hi) return;
    {
        const ColRec pc = cols[c_first - base - 1];
        float2 S[R / 2];
        float Ss;
        sq_packed<R>(rb, pc, S, Ss);
#pragma unroll
        for (int m = 0; m < R / 2; ++m) rb.Sp[m] = S[m];
    }
    uint32_t c = c_first;
    while (c < c_hi) {
        const uint32_t w = (c - wbase) / kWin;
        const uint32_t wend = min(c_hi, wbase + (w + 1) * kWin);
        const float emax = wmax[w];
        window_thresholds<R>(rb, emax);
        const uint32_t peel_end = min(wend, ib + R + 1);
        for (; c < peel_end; ++c)
            column_step4<R, true>(rb, cols, base, c, ib, n, Q, emax, B, best);
#pragma unroll 2
        for (; c < wend; ++c)
            column_step4<R, false>(rb, cols, base, c, ib, n, Q, emax, B, best);
    }
}

}  // namespace logo
