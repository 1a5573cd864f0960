// Local-coordinate expanded screen of the sweep (LOGO_SWEEP_LOCAL).
//
// A pair (i, c) can only be chosen if d1 = nint d(i, c) <= V = B + e[i] +
// e[c] (B <= -1 the best exact delta known; see sweep_core5.cuh).  Here the
// test on d(i, c) is rewritten around an origin o (the coordinates of the
// tile's first row), with a, b the row's and p, q the column's coordinates
// relative to o (each one binary32 subtraction):
//     |r - q|^2 - |r|^2 = |q|^2 - 2 a p - 2 b q
//     v = RN(-2b * q + RN(-2a * p + C)),  C = RN(q*q + RN(p*p))   (per column)
// and row i passes in column c when v < T_i, with the per-row threshold
//     T_i = RN(RN(L - RN(b*b + RN(a*a))) + m),  L = RN(u*u),
//     m = 2^-18 (|a| + |b| + u)^2,  u = B + e[i] + 5 + E
// (E = the largest e over the column window; u <= 0 means no pair of the row
// can pass and T = -FLT_MAX).  Per pair that is two FFMA lane operations,
// issued as FFMA2 over two adjacent columns (the per-column p, q, C are read
// as float4 from a structure-of-arrays tile), and one third of a three-input
// min (the row's minimum v over a group of columns is compared with T once
// per group).  Columns of a group with a passing row then go through the
// stages of sweep_core5.cuh: d(i-1, c-1) against the row's L, the per-pair
// squared test with the exact e[c], and the exact distances.
//
// Why no chosen pair is missed (every quantity is finite; V >= 0, else no
// pair can be chosen).  Let X = x_i - x_c, Y = y_i - y_c (real).  As in
// sweep_core5.cuh the reference distance satisfies d1 <= V only if
// X^2 + Y^2 < (V + 0.5)^2 (1 + 2^-21).  The local differences are
// a - p = X + alpha - pi with |alpha| <= 2^-24 |a|, |pi| <= 2^-24 |p| (and
// the same in y), so D = |(a - p, b - q)| <= |(X, Y)| + 2^-24 S (1 + 2^-20),
// S = |a| + |b| + |p| + |q| <= 2 (rho + u), rho = |a| + |b| (because
// |p| + |q| <= rho + sqrt(2) D and D <= V + 2, u >= V + 5).  Exactly,
// D^2 - (a^2 + b^2) = W = p^2 + q^2 - 2ap - 2bq; every term and every
// partial sum of the evaluation of v is at most S^2 in magnitude, and there
// are four roundings (two in C counted at 2^-23, one per FFMA), so
// |v - W| <= 5.1 * 2^-24 S^2 <= 20.4 * 2^-24 (rho + u)^2.  Hence
//     v <= (V + 0.5)^2 - (a^2 + b^2) + 32.4 * 2^-24 (rho + u)^2.
// The threshold before rounding is L - (a^2 + b^2) + 64 * 2^-24 (rho + u)^2
// with L >= (V + 5)^2 (1 - 2^-24) > (V + 0.5)^2 + 2^-24 u^2; computing it
// (a^2 + b^2 to 2^-23, two more roundings, m itself) loses at most
// 4.5 * 2^-24 (rho + u)^2.  So T exceeds the bound on v by more than
// 27 * 2^-24 (rho + u)^2 > 0 and v < T for every pair that can be chosen.
// The origin keeps rho small for rows near it (a tile of consecutive tour
// positions is usually spatially compact), so the margin m stays far below
// the spacing of neighbouring cities; rows far from it only get a looser
// (still exact-checked) screen.
#pragma once
#include <cfloat>
#include "sweep_core5.cuh"

namespace logo {

constexpr uint32_t kWin6 = 32;
constexpr float kMargin6 = 3.814697265625e-6f;  // 2^-18

__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

template <int R>
struct RowBlock6 {
    float gx[R + 1], gy[R + 1];  // global coordinates of rows ib - 1 + k, k = 0..R
    float2 ax2[R], by2[R];       // (-2a, -2a), (-2b, -2b) of pair row r (row ib + r)
    float T2[R];                 // B + e[ib + r] + 5, or -3e7 for rows without pairs
    float T[R];                  // stage-1 threshold for the current window
    float NL[R];                 // -L of pair row r for the current window (stage 2)
    float4 rbox;                 // bounding box (x0, x1, y0, y1) of the R pair rows
    float T2max;                 // max over r of T2[r]
};

template <int R>
__device__ __forceinline__ void load_rows6(RowBlock6<R>& rb, const OrderedCity* Q, uint32_t ib,
                                           uint32_t n, float ox, float oy) {
#pragma unroll
    for (int k = 0; k <= R; ++k) {
        const OrderedCity z = Q[min(ib - 1 + k, n - 1)];
        rb.gx[k] = z.x;
        rb.gy[k] = z.y;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float a = __fsub_rn(rb.gx[r + 1], ox), b = __fsub_rn(rb.gy[r + 1], oy);
        rb.ax2[r] = make_float2(-2.f * a, -2.f * a);
        rb.by2[r] = make_float2(-2.f * b, -2.f * b);
    }
}

template <int R>
__device__ __forceinline__ void refresh6(RowBlock6<R>& rb, const OrderedCity* Q, uint32_t ib,
                                         uint32_t n, int B) {
    rb.T2max = -3.0e7f;
    rb.rbox = make_float4(rb.gx[1], rb.gx[1], rb.gy[1], rb.gy[1]);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        rb.T2[r] = (i + 3 <= n) ? (float)(B + (int)Q[i].e + 5) : -3.0e7f;
        rb.T2max = fmaxf(rb.T2max, rb.T2[r]);
        rb.rbox.x = fminf(rb.rbox.x, rb.gx[r + 1]);
        rb.rbox.y = fmaxf(rb.rbox.y, rb.gx[r + 1]);
        rb.rbox.z = fminf(rb.rbox.z, rb.gy[r + 1]);
        rb.rbox.w = fmaxf(rb.rbox.w, rb.gy[r + 1]);
    }
}

// Thresholds of the current window (largest edge emax).
template <int R>
__device__ __forceinline__ void window6(RowBlock6<R>& rb, float emax) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float u = rb.T2[r] + emax;
        const float a2 = rb.ax2[r].x, b2 = rb.by2[r].x;  // -2a, -2b (exact)
        const float rho = 0.5f * (fabsf(a2) + fabsf(b2));
        const float rho2 = 0.25f * __fmaf_rn(b2, b2, __fmul_rn(a2, a2));  // RN(b^2 + RN(a^2))
        const float L = __fmul_rn(u, u);
        const float s = rho + u;
        const float m = kMargin6 * __fmul_rn(s, s);
        rb.T[r] = u > 0.f ? __fadd_rn(__fsub_rn(L, rho2), m) : -FLT_MAX;
        rb.NL[r] = u > 0.f ? -L : 0.f;
    }
}

template <int R>
__device__ __forceinline__ void lower_b6(RowBlock6<R>& rb, int& B, int g) {
    const float shift = (float)(g - B);
#pragma unroll
    for (int r = 0; r < R; ++r) rb.T2[r] += shift;
    rb.T2max += shift;
    B = g;
}

// Column tile in shared memory: cx[j], cy[j], cc[j] = p, q, C of column
// col0 + j; stg[j + 1] = column col0 + j (stg[0] = column col0 - 1).
struct ColTile6 {
    const float* cx;
    const float* cy;
    const float* cc;
    const OrderedCity* stg;
};

// Stages 2 and 3 for the rows in `rows` (stage 1 passed) of column c
// (tile index j).
template <int R>
__device__ __forceinline__ void column_rest6(RowBlock6<R>& rb, uint32_t rows, const ColTile6& t,
                                             uint32_t j, uint32_t c, uint32_t ib, float emax,
                                             Best5& bs) {
    const OrderedCity q = t.stg[j + 1], qp = t.stg[j];
    uint32_t rows2 = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float dx = __fsub_rn(rb.gx[r], qp.x), dy = __fsub_rn(rb.gy[r], qp.y);
        const float t2 = __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, rb.NL[r]));
        rows2 |= (__float_as_uint(t2) >> 31) << r;
    }
    rows2 &= rows;
    if (!rows2) return;
    const int ec = (int)q.e;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!((rows2 >> r) & 1u)) continue;
        const uint32_t i = ib + r;
        const float xr = rb.gx[r + 1], yr = rb.gy[r + 1];
        const float xq = rb.gx[r], yq = rb.gy[r];
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
                    lower_b6<R>(rb, bs.B, delta);
                    window6<R>(rb, emax);
                }
            }
        }
    }
}

// One column, all stages; MASK drops pairs with c < i + 2.
template <int R, bool MASK>
__device__ __forceinline__ void column6(RowBlock6<R>& rb, const ColTile6& t, uint32_t j,
                                        uint32_t c, uint32_t ib, float emax, Best5& bs) {
    const float p = t.cx[j], q = t.cy[j], C = t.cc[j];
    uint32_t rows = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float v = __fmaf_rn(rb.by2[r].x, q, __fmaf_rn(rb.ax2[r].x, p, C));
        const bool ok = v < rb.T[r] && (!MASK || c >= ib + r + 2);
        rows |= (uint32_t)ok << r;
    }
    if (rows) {
        bs.busy = true;
        column_rest6<R>(rb, rows, t, j, c, ib, emax, bs);
    }
}

// Stage 1 over G columns starting at tile index j (j % 4 == 0): true when
// some row passes in some column.
template <int R, int G>
__device__ __forceinline__ bool group6(const RowBlock6<R>& rb, const ColTile6& t, uint32_t j) {
    const float4* px = reinterpret_cast<const float4*>(t.cx + j);
    const float4* py = reinterpret_cast<const float4*>(t.cy + j);
    const float4* pc = reinterpret_cast<const float4*>(t.cc + j);
    float acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = FLT_MAX;
#pragma unroll
    for (int g = 0; g < G / 4; ++g) {
        const float4 P = px[g], Qv = py[g], Cv = pc[g];
        const float2 p0 = make_float2(P.x, P.y), p1 = make_float2(P.z, P.w);
        const float2 q0 = make_float2(Qv.x, Qv.y), q1 = make_float2(Qv.z, Qv.w);
        const float2 c0 = make_float2(Cv.x, Cv.y), c1 = make_float2(Cv.z, Cv.w);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float2 v0 = __ffma2_rn(rb.by2[r], q0, __ffma2_rn(rb.ax2[r], p0, c0));
            const float2 v1 = __ffma2_rn(rb.by2[r], q1, __ffma2_rn(rb.ax2[r], p1, c1));
            acc[r] = min3f(acc[r], v0.x, v0.y);
            acc[r] = min3f(acc[r], v1.x, v1.y);
        }
    }
    bool pass = false;
#pragma unroll
    for (int r = 0; r < R; ++r) pass |= acc[r] < rb.T[r];
    return pass;
}

// Window test of the boxed screen (LOGO_SWEEP_BOXED): box = (X0, X1, Y0, Y1),
// the bounding box of the window's column coordinates (global binary32
// values).  Rows that cannot be chosen in any column of the window get
// T = -FLT_MAX; false when no row of the thread is left.
//
// Why no chosen pair is missed.  For a column c of the window and row i at
// (x, y), |x - x_c| >= gx where gx is the real gap between x and [X0, X1]
// (0 inside), and the gap is one exact binary32 difference (X0 - x or
// x - X1), so rounding is monotone: |RN(x - x_c)| >= RN(gx).  The reference
// squares dx = RN(x - x_c), dy = RN(y - y_c); with s = RN(gy^2 + RN(gx^2))
// (two roundings, each up by at most 2^-24 relative),
// dx^2 + dy^2 >= s (1 + 2^-24)^-2.  A chosen pair needs
// dx^2 + dy^2 < (V + 0.5)^2 (1 + 2^-22) (sweep_core5.cuh), so
// s < (V + 0.5)^2 (1 + 2^-21) <= (V + 5)^2 (1 - 2^-24) <= L for every
// V < 1.6e7 (here V < 4e6), L = RN(u^2) the row's stage-2 threshold of the
// window (u >= V + 5).  Rows with u <= 0 have L = 0 and fail s < L.  Lowering
// B later in the window only tightens the thresholds (window6 recomputes T
// for every row; the rows this test removed then pass through stage 1 again,
// which costs work but changes no result).
// The same test for the thread's rows together, before any per-row work:
// every row lies in rb.rbox, so the gap between the two boxes (again one
// exact binary32 difference per axis) bounds every |RN(x - x_c)|, and
// u = T2max + E bounds every row's u.
template <int R>
__device__ __forceinline__ bool box_block6(const RowBlock6<R>& rb, float4 box, float emax) {
    const float u = rb.T2max + emax;
    const float gx = fmaxf(fmaxf(__fsub_rn(box.x, rb.rbox.y), __fsub_rn(rb.rbox.x, box.y)), 0.f);
    const float gy = fmaxf(fmaxf(__fsub_rn(box.z, rb.rbox.w), __fsub_rn(rb.rbox.z, box.w)), 0.f);
    const float s = __fmaf_rn(gy, gy, __fmul_rn(gx, gx));
    return u > 0.f && s < __fmul_rn(u, u);
}

template <int R>
__device__ __forceinline__ bool box_rows6(RowBlock6<R>& rb, float4 box) {
    bool any = false;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const float x = rb.gx[r + 1], y = rb.gy[r + 1];
        const float gx = fmaxf(fmaxf(__fsub_rn(box.x, x), __fsub_rn(x, box.y)), 0.f);
        const float gy = fmaxf(fmaxf(__fsub_rn(box.z, y), __fsub_rn(y, box.w)), 0.f);
        const float s = __fmaf_rn(gy, gy, __fmul_rn(gx, gx));
        const bool ok = s < -rb.NL[r];
        rb.T[r] = ok ? rb.T[r] : -FLT_MAX;
        any |= ok;
    }
    return any;
}

// Walks columns [c_lo, c_hi) of the tile whose first column is col0.
// wmax[w] = largest e over columns [col0 + w*kWin6, col0 + (w+1)*kWin6) and,
// with BOX, wbox[w] = the bounding box of their coordinates (both in global
// memory) and mask = the windows whose box test passed at the start: the
// others, and those whose test fails with the current B, are skipped.
// Sharing of B between threads as in walk_columns5.
template <int R, int G, bool BOX>
__device__ __forceinline__ void walk_columns6(RowBlock6<R>& rb, const ColTile6& t,
                                              const float* wmax, const float4* wbox,
                                              uint32_t mask, uint32_t col0, uint32_t c_lo,
                                              uint32_t c_hi, uint32_t ib, uint32_t n,
                                              DevState* st, Best5& bs) {
    static_assert(G % 4 == 0 && kWin6 % G == 0, "groups are float4-aligned inside windows");
    const uint32_t c_first = max(c_lo, ib + 2);
    if (ib + 3 > n || c_first >= c_hi) return;
    uint32_t c = c_first;
    uint64_t gk = kNoMove;  // read at the end of the previous window
    while (c < c_hi) {
        uint32_t w = (c - col0) / kWin6;
        if (BOX) {  // next window of the mask (earlier windows stay published)
            const uint32_t rest = w < 32 ? (mask >> w) : 0u;
            if (!rest) break;
            w += __ffs(rest) - 1;
            c = max(c, col0 + w * kWin6);
        }
        const uint32_t wend = min(c_hi, col0 + (w + 1) * kWin6);
        const float emax = BOX ? __ldg(wmax + w) : wmax[w];
        bs.busy = false;
        bool open = true;
        if (BOX) {
            const float4 box = __ldg(wbox + w);
            open = box_block6<R>(rb, box, emax);
            if (open) {
                window6<R>(rb, emax);
                open = box_rows6<R>(rb, box);
            }
        } else {
            window6<R>(rb, emax);
        }
        if (open) {
            const uint32_t peel_end = min(wend, ib + R + 1);
            for (; c < peel_end; ++c) column6<R, true>(rb, t, c - col0, c, ib, emax, bs);
            for (; c < wend && ((c - col0) & 3u); ++c)
                column6<R, false>(rb, t, c - col0, c, ib, emax, bs);
            for (; c + G <= wend; c += G) {
                if (group6<R, G>(rb, t, c - col0)) {
                    bs.busy = true;
#pragma unroll 1
                    for (uint32_t k = 0; k < G; ++k)
                        column6<R, false>(rb, t, c + k - col0, c + k, ib, emax, bs);
                }
            }
            for (; c < wend; ++c) column6<R, false>(rb, t, c - col0, c, ib, emax, bs);
        }
        c = wend;
        if (bs.B < bs.G) {
            atomicMin(&st->best_key, (unsigned long long)bs.best);
            bs.G = bs.B;
        }
        if (gk != kNoMove) {
            const int g = key_delta(gk);
            if (g < bs.B) lower_b6<R>(rb, bs.B, g);
            if (g < bs.G) bs.G = g;
        }
        gk = bs.busy ? *(volatile unsigned long long*)&st->best_key : kNoMove;
    }
}

}  // namespace logo
