// Fused square-root-free screen of the sweep (LOGO_SWEEP_FUSED).
//
// A pair (i, c) can only be chosen if its exact delta is <= B, the best exact
// delta known (B <= -1).  With d1 = nint d(i, c), d2 = nint d(i-1, c-1) >= 0
// that needs d1 <= V and d2 <= V, V = B + e[i] + e[c].  The screen tests
// them in two stages, with the threshold folded into the sum of squares:
//     t = RN(dy*dy + RN(dx*dx - L_r)),  L_r = RN(u*u),  u = B + e[i] + 5 + E,
// E = the largest e over a window of kWin5 columns (E >= e[c]).
//   stage 1, every column: t of d(i, c) for the thread's R rows, two rows per
//     FADD2 / FADD2 / FFMA2 / FFMA2, and an OR of the sign bits;
//   stage 2, only when some row passed stage 1: t of d(i-1, c-1) for the
//     passing rows (scalar), ANDed with stage 1's bits;
//   stage 3, only when a row passed both: the per-pair test of
//     sweep_core3.cuh (max(s(i, c), s(i-1, c-1)) < RN(u |u|) with the exact
//     e[c]) and the exact distances.
// Stage 1 is 4 lane operations per pair and needs neither the row i-1 entry
// nor the previous column; stage 2 removes the columns that only one end of
// a long incoming edge is near.
//
// Why no chosen pair is missed.  dx, dy are the binary32 differences the
// reference squares; write a = dx^2, b = dy^2 (real numbers) and
// s = RN(RN(a) + RN(b)) for the reference's binary32 sum.  The reference
// distance is trunc(RN(RN(sqrt(s)) + 0.5)); since V + 0.5 and V + 1 are
// binary32 numbers (0 <= V < 2^23), d <= V implies sqrt(s) < V + 0.5, so
// s < (V + 0.5)^2 and a + b <= s (1 - 2^-24)^-2 < (V + 0.5)^2 (1 + 2^-22).
// With u >= V + 5 > 0, L >= (V + 5)^2 (1 - 2^-24).  Rounding the negative
// a - L moves it by at most 2^-24 L towards zero and FFMA rounds once, so
// b + RN(a - L) <= a + b - L (1 - 2^-24), negative whenever
// (V + 0.5)^2 (1 + 2^-22) < (V + 5)^2 (1 - 2^-24)^2, i.e. whenever
// 9 / (V + 0.5) > 3.6e-7: every V < 2.5e7 (here V < 4e6, the coordinate box
// diagonal being below 2e6).  A negative sum rounds to a negative number or
// to -0 (flushing keeps the sign), so its sign bit is set.  For u <= 0 (no
// pair of that row can pass) L is taken as 0, and t >= +0.  Lowering B (own
// finds, or the best delta other threads have published) only tightens the
// thresholds.  The chosen move is the exact lowest
// (delta, i, c): every pair with exact delta <= B reaches stage 3.
#pragma once
#include "sweep_core3.cuh"

namespace logo {

constexpr uint32_t kWin5 = 32;

template <int R>
struct RowBlock5 {
    float2 x[R / 2], y[R / 2];  // rows ib + 2m, ib + 2m + 1 (pair rows 2m, 2m + 1)
    float xp, yp;               // row ib - 1
    float T2[R];                // B + e[ib + r] + 5, or -3e7 for rows without pairs
    float2 NL[R / 2];           // -L of pair rows 2m, 2m + 1 for the current window
};

template <int R>
__device__ __forceinline__ void load_rows5(RowBlock5<R>& rb, const OrderedCity* Q, uint32_t ib,
                                           uint32_t n) {
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const OrderedCity a = Q[min(ib + 2 * m, n - 1)], b = Q[min(ib + 2 * m + 1, n - 1)];
        rb.x[m] = make_float2(a.x, b.x);
        rb.y[m] = make_float2(a.y, b.y);
    }
    const OrderedCity z = Q[min(ib - 1, n - 1)];
    rb.xp = z.x;
    rb.yp = z.y;
}

template <int R>
__device__ __forceinline__ void refresh5(RowBlock5<R>& rb, const OrderedCity* Q, uint32_t ib,
                                         uint32_t n, int B) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        rb.T2[r] = (i + 3 <= n) ? (float)(B + (int)Q[i].e + 5) : -3.0e7f;
    }
}

// -L = -(max(u, 0) * u): u > 0 gives -RN(u^2); u <= 0 gives +0 (never passes).
template <int R>
__device__ __forceinline__ void window_nl5(RowBlock5<R>& rb, float emax) {
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const float u0 = rb.T2[2 * m] + emax, u1 = rb.T2[2 * m + 1] + emax;
        rb.NL[m] = make_float2(-(fmaxf(u0, 0.f) * u0), -(fmaxf(u1, 0.f) * u1));
    }
}

// Lowers B to g (g < B), keeping T2 = B + e + 5 exact.
template <int R>
__device__ __forceinline__ void lower_b5(RowBlock5<R>& rb, int& B, int g) {
    const float shift = (float)(g - B);
#pragma unroll
    for (int r = 0; r < R; ++r) rb.T2[r] += shift;
    B = g;
}

// Row r of the block (r = -1: row ib - 1).
template <int R>
__device__ __forceinline__ float row_x5(const RowBlock5<R>& rb, int r) {
    return r < 0 ? rb.xp : ((r & 1) ? rb.x[r >> 1].y : rb.x[r >> 1].x);
}
template <int R>
__device__ __forceinline__ float row_y5(const RowBlock5<R>& rb, int r) {
    return r < 0 ? rb.yp : ((r & 1) ? rb.y[r >> 1].y : rb.y[r >> 1].x);
}
template <int R>
__device__ __forceinline__ float row_nl5(const RowBlock5<R>& rb, int r) {
    return (r & 1) ? rb.NL[r >> 1].y : rb.NL[r >> 1].x;
}

struct Best5 {
    uint64_t best;     // lowest key this thread has found
    int B;             // best exact delta known (own or published)
    int G;             // best delta this thread has published or read
    bool busy;         // stage 2 ran in the current window
    float M;           // bound on |exact - approximate delta| (filter_margin of the instance)
};

// Last test before the exact distances of a pair that passed the squared
// screens: the approximate delta (contracted sums of squares, MUFU square
// roots) against B + M, in the MUFU screen's own form and rounding order
// (sweep_core.cuh), whose margin M = filter_margin(diag) bounds |exact delta
// - approximate delta| for every pair.  A pair whose exact delta is <= B
// always passes; the squared screens test each distance against V = B +
// e[i] + e[c] on its own, this one their sum, which is what removes most
// exact evaluations where long edges make V large.
__device__ __forceinline__ bool approx_delta_pass(float xr, float yr, float xq, float yq,
                                                  const OrderedCity& q, const OrderedCity& qp,
                                                  int ei, int B, float M) {
    const float v = approx_dist(xr, yr, q.x, q.y) + (approx_dist(xq, yq, qp.x, qp.y) - q.e);
    return v < (float)(B + ei) + M;
}

// Stage 3 for the rows whose bit is set in `rows`: per-pair squared test with
// the exact e[c], then the exact delta.  q = column c, qp = column c - 1.
template <int R>
__device__ __forceinline__ void column_exact5(RowBlock5<R>& rb, uint32_t rows,
                                              const OrderedCity& q, const OrderedCity& qp,
                                              uint32_t c, uint32_t ib, float emax, Best5& bs) {
    const int ec = (int)q.e;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!((rows >> r) & 1u)) continue;
        const uint32_t i = ib + r;
        const float xr = row_x5<R>(rb, r), yr = row_y5<R>(rb, r);
        const float xq = row_x5<R>(rb, r - 1), yq = row_y5<R>(rb, r - 1);
        const float u = rb.T2[r] + q.e;
        const float L = u * fabsf(u);
        const int ei = (int)rb.T2[r] - bs.B - 5;  // rows that reach here have pairs
        if (fmaxf(sq_dist(xr, yr, q.x, q.y), sq_dist(xq, yq, qp.x, qp.y)) < L &&
            approx_delta_pass(xr, yr, xq, yq, q, qp, ei, bs.B, bs.M)) {
            const int d1 = exact_dist(xr, yr, q.x, q.y);
            const int d2 = exact_dist(xq, yq, qp.x, qp.y);
            const int delta = d1 + d2 - ei - ec;
            if (delta <= bs.B) {
                const uint64_t key = pack_key(delta, i, c);
                bs.best = key < bs.best ? key : bs.best;
                if (delta < bs.B) {
                    lower_b5<R>(rb, bs.B, delta);
                    window_nl5<R>(rb, emax);
                }
            }
        }
    }
}

// Stage 1 of one column, sign bits ORed over the R rows (no masking).
template <int R>
__device__ __forceinline__ uint32_t stage1_any5(const RowBlock5<R>& rb, const float4 h) {
    const float2 qx = make_float2(h.x, h.y), qy = make_float2(h.z, h.w);
    uint32_t acc = 0;
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const float2 dx = __fadd2_rn(rb.x[m], qx);
        const float2 dy = __fadd2_rn(rb.y[m], qy);
        const float2 t = __ffma2_rn(dy, dy, __ffma2_rn(dx, dx, rb.NL[m]));
        acc |= __float_as_uint(t.x) | __float_as_uint(t.y);
    }
    return acc;
}

// hot[c - base] = (-x, -x, -y, -y) and stg[c - base] = column c.
template <int R, bool MASK>
__device__ __forceinline__ void column_step5(RowBlock5<R>& rb, const float4* hot,
                                             const OrderedCity* stg, uint32_t base, uint32_t c,
                                             uint32_t ib, float emax, Best5& bs) {
    const float4 h = hot[c - base];
    const float2 qx = make_float2(h.x, h.y), qy = make_float2(h.z, h.w);
    uint32_t T[R];
    uint32_t acc = 0;
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const float2 dx = __fadd2_rn(rb.x[m], qx);
        const float2 dy = __fadd2_rn(rb.y[m], qy);
        const float2 t = __ffma2_rn(dy, dy, __ffma2_rn(dx, dx, rb.NL[m]));
        T[2 * m] = __float_as_uint(t.x);
        T[2 * m + 1] = __float_as_uint(t.y);
        if (MASK) {
            T[2 * m] = (c >= ib + 2 * m + 2) ? T[2 * m] : 0u;
            T[2 * m + 1] = (c >= ib + 2 * m + 3) ? T[2 * m + 1] : 0u;
        }
        acc |= T[2 * m] | T[2 * m + 1];
    }
    if ((int)acc < 0) {
        bs.busy = true;
        // stage 2: d(i-1, c-1) against the same row thresholds
        const float4 hp = hot[c - 1 - base];
        uint32_t rows = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float dx = __fadd_rn(row_x5<R>(rb, r - 1), hp.x);
            const float dy = __fadd_rn(row_y5<R>(rb, r - 1), hp.z);
            const float t = __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, row_nl5<R>(rb, r)));
            rows |= ((T[r] & __float_as_uint(t)) >> 31) << r;
        }
        if (rows) column_exact5<R>(rb, rows, stg[c - base], stg[c - base - 1], c, ib, emax, bs);
    }
}

// wmax[w] = largest e over columns [wbase + w*kWin5, wbase + (w+1)*kWin5).
//
// Sharing B between threads: at the end of a window a thread publishes a new
// best of its own (atomicMin on the sweep's key), and a thread whose screen
// let something through in that window reads the published best; the value
// is applied at the end of the next window, so the read's latency is hidden.
// Threads whose screens pass nothing do not poll.  G > 1 evaluates stage 1
// for G columns before one branch (fewer branches and reconvergence points
// per column; better when few columns pass, i.e. on large tours).
template <int R, int G>
__device__ __forceinline__ void walk_columns5(RowBlock5<R>& rb, const float4* hot,
                                              const OrderedCity* stg, uint32_t base,
                                              const float* wmax, uint32_t wbase, uint32_t c_lo,
                                              uint32_t c_hi, uint32_t ib, uint32_t n,
                                              DevState* st, Best5& bs) {
    const uint32_t c_first = max(c_lo, ib + 2);
    if (ib + 3 > n || c_first >= c_hi) return;
    uint32_t c = c_first;
    uint64_t gk = kNoMove;  // read at the end of the previous window
    while (c < c_hi) {
        const uint32_t w = (c - wbase) / kWin5;
        const uint32_t wend = min(c_hi, wbase + (w + 1) * kWin5);
        const float emax = wmax[w];
        window_nl5<R>(rb, emax);
        bs.busy = false;
        const uint32_t peel_end = min(wend, ib + R + 1);
        for (; c < peel_end; ++c) column_step5<R, true>(rb, hot, stg, base, c, ib, emax, bs);
        if (G > 1) {
            // groups of G columns share one branch; in a group where some row
            // passes stage 1, the passing columns are redone one by one
            for (; c + G <= wend; c += G) {
                uint32_t acc[G];
#pragma unroll
                for (int j = 0; j < G; ++j) acc[j] = stage1_any5<R>(rb, hot[c + j - base]);
                uint32_t any = 0;
#pragma unroll
                for (int j = 0; j < G; ++j) any |= acc[j];
                if ((int)any < 0) {
                    uint32_t pass = 0;
#pragma unroll
                    for (int j = 0; j < G; ++j) pass |= (acc[j] >> 31) << j;
                    while (pass) {
                        const uint32_t j = __ffs(pass) - 1;
                        pass &= pass - 1;
                        column_step5<R, false>(rb, hot, stg, base, c + j, ib, emax, bs);
                    }
                }
            }
        }
#pragma unroll 4
        for (; c < wend; ++c) column_step5<R, false>(rb, hot, stg, base, c, ib, emax, bs);
        if (bs.B < bs.G) {
            atomicMin(&st->best_key, (unsigned long long)bs.best);
            bs.G = bs.B;
        }
        if (gk != kNoMove) {
            const int g = key_delta(gk);
            if (g < bs.B) lower_b5<R>(rb, bs.B, g);
            if (g < bs.G) bs.G = g;
        }
        gk = bs.busy ? *(volatile unsigned long long*)&st->best_key : kNoMove;
    }
}

}  // namespace logo
