// Packed (f32x2) variant of the per-thread sweep core for sm_100-class GPUs.
//
// Same candidate set, filter and exact re-evaluation as sweep_core.cuh; the
// difference is how the fast path is issued.  Rows are held in register
// pairs (x[2m], x[2m+1]) and a column is read as broadcast pairs
// (x, x), (y, y), (e, e) from a 32-byte shared-memory record, so that the
// difference, square and sum of squares of two distances are one FFMA2 /
// FMUL2 / FFMA2 each:
//     d = q * (-1) + r          (x and y, two rows at once)
//     s = dy * dy + dx * dx
//     D = sqrt.approx(s)        (one MUFU per distance)
// and the filter test for pair row r becomes
//     D(r+1, c) < Z[r],  Z = (T + e_c) - D(r, c-1)
// with Z formed for two rows per FADD2 / FFMA2.  Per column: R+1 distances,
// (R/2)*4 + 4 packed/scalar FP instructions, R+1 MUFU, R compares.
#pragma once
#include "sweep_core.cuh"

namespace logo {

// Column record in shared memory: broadcast pairs.
struct __align__(32) ColRec {
    float2 x;  // (x, x)
    float2 y;  // (y, y)
    float2 e;  // (e, e)
    float2 xy; // (x, y) for the exact path
};

__device__ __forceinline__ ColRec make_colrec(const OrderedCity& c) {
    ColRec r;
    r.x = make_float2(c.x, c.x);
    r.y = make_float2(c.y, c.y);
    r.e = make_float2(c.e, c.e);
    r.xy = make_float2(c.x, c.y);
    return r;
}

__device__ __forceinline__ float sqrt_approx(float s) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s));
    return r;
}

// R even.  Rows ib-1 .. ib+R-1: packs m = 0 .. R/2-1 hold rows (2m, 2m+1)
// (k = row - (ib-1)), row k = R is single.
template <int R>
struct RowBlock2 {
    float2 x[R / 2], y[R / 2];
    float xs, ys;        // row k = R
    float2 T[R / 2];     // thresholds of pair rows (2m, 2m+1)
    float2 Dp[R / 2];    // approx d(row k, c-1), k = 0..R-1
};

template <int R>
__device__ __forceinline__ void load_rows2(RowBlock2<R>& rb, const OrderedCity* Q, uint32_t ib,
                                           uint32_t n) {
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const uint32_t i0 = min(ib - 1 + 2 * m, n - 1), i1 = min(ib + 2 * m, n - 1);
        const OrderedCity a = Q[i0], b = Q[i1];
        rb.x[m] = make_float2(a.x, b.x);
        rb.y[m] = make_float2(a.y, b.y);
    }
    const OrderedCity z = Q[min(ib - 1 + R, n - 1)];
    rb.xs = z.x;
    rb.ys = z.y;
}

template <int R>
__device__ __forceinline__ void refresh_thresholds2(RowBlock2<R>& rb, const OrderedCity* Q,
                                                    uint32_t ib, uint32_t n, int B, float margin) {
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        float t[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t i = ib + 2 * m + h;
            t[h] = (i + 3 <= n) ? (float)(B + (int)Q[i].e) + margin : -INFINITY;
        }
        rb.T[m] = make_float2(t[0], t[1]);
    }
}

template <int R>
__device__ __forceinline__ float row_x(const RowBlock2<R>& rb, int k) {
    return k == R ? rb.xs : ((k & 1) ? rb.x[k >> 1].y : rb.x[k >> 1].x);
}
template <int R>
__device__ __forceinline__ float row_y(const RowBlock2<R>& rb, int k) {
    return k == R ? rb.ys : ((k & 1) ? rb.y[k >> 1].y : rb.y[k >> 1].x);
}
__device__ __forceinline__ float pair_of(const float2* v, int k) {
    return (k & 1) ? v[k >> 1].y : v[k >> 1].x;
}

// Approximate distances of the R+1 rows to column q: Dc packs + single.
template <int R>
__device__ __forceinline__ void distances2(const RowBlock2<R>& rb, const ColRec& q, float2* Dc,
                                           float& Ds) {
    const float2 neg1 = make_float2(-1.f, -1.f);
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const float2 dx = __ffma2_rn(q.x, neg1, rb.x[m]);
        const float2 dy = __ffma2_rn(q.y, neg1, rb.y[m]);
        float2 s = __fmul2_rn(dx, dx);
        s = __ffma2_rn(dy, dy, s);
        Dc[m] = make_float2(sqrt_approx(s.x), sqrt_approx(s.y));
    }
    const float dxs = rb.xs - q.x.x, dys = rb.ys - q.y.x;
    Ds = sqrt_approx(__fmaf_rn(dys, dys, dxs * dxs));
}

// The filter value of pair row r at column c: D(r+1, c) < Z[r].
template <int R>
__device__ __forceinline__ void column_exact2(RowBlock2<R>& rb, const float2* Dc, float Ds,
                                              const ColRec& q, const ColRec& qp, uint32_t c,
                                              uint32_t ib, uint32_t n, const OrderedCity* Q,
                                              float margin, int& B, uint64_t& best) {
    const int ec = (int)q.e.x;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t i = ib + r;
        const float dcur = (r + 1 == R) ? Ds : pair_of(Dc, r + 1);
        const float z = (pair_of(rb.T, r) + q.e.x) - pair_of(rb.Dp, r);
        if (c >= i + 2 && dcur < z) {
            const int d1 = exact_dist(row_x<R>(rb, r + 1), row_y<R>(rb, r + 1), q.xy.x, q.xy.y);
            const int d2 = exact_dist(row_x<R>(rb, r), row_y<R>(rb, r), qp.xy.x, qp.xy.y);
            const int ei = (int)Q[i].e;
            const int delta = d1 + d2 - ei - ec;
            if (delta <= B) {
                const uint64_t key = pack_key(delta, i, c);
                best = key < best ? key : best;
                if (delta < B) {
                    B = delta;
                    refresh_thresholds2<R>(rb, Q, ib, n, B, margin);
                }
            }
        }
    }
}

template <int R, bool MASK>
__device__ __forceinline__ void column_step2(RowBlock2<R>& rb, const ColRec* cols, uint32_t base,
                                             uint32_t c, uint32_t ib, uint32_t n,
                                             const OrderedCity* Q, float margin, int& B,
                                             uint64_t& best) {
    const ColRec q = cols[c - base];
    float2 Dc[R / 2];
    float Ds;
    distances2<R>(rb, q, Dc, Ds);
    const float2 neg1 = make_float2(-1.f, -1.f);
    bool hit = false;
#pragma unroll
    for (int m = 0; m < R / 2; ++m) {
        const float2 te = __fadd2_rn(rb.T[m], q.e);
        const float2 z = __ffma2_rn(rb.Dp[m], neg1, te);
        // pair rows 2m, 2m+1 compare D(2m+1) and D(2m+2)
        const float d0 = Dc[m].y;
        const float d1 = (m + 1 < R / 2) ? Dc[m + 1].x : Ds;
        bool c0 = d0 < z.x, c1 = d1 < z.y;
        if (MASK) {
            c0 = c0 && (c >= ib + 2 * m + 2);
            c1 = c1 && (c >= ib + 2 * m + 3);
        }
        hit |= c0 | c1;
    }
    if (hit) {
        const ColRec qp = cols[c - base - 1];
        column_exact2<R>(rb, Dc, Ds, q, qp, c, ib, n, Q, margin, B, best);
    }
#pragma unroll
    for (int m = 0; m < R / 2; ++m) rb.Dp[m] = Dc[m];
}

template <int R>
__device__ __forceinline__ void walk_columns2(RowBlock2<R>& rb, const ColRec* cols, uint32_t base,
                                              uint32_t c_lo, uint32_t c_hi, uint32_t ib,
                                              uint32_t n, const OrderedCity* Q, float margin,
                                              int& B, uint64_t& best) {
    const uint32_t c_first = max(c_lo, ib + 2);
    if (ib + 3 > n || c_first >= c_hi) return;
    {
        const ColRec pc = cols[c_first - base - 1];
        float2 Dc[R / 2];
        float Ds;
        distances2<R>(rb, pc, Dc, Ds);
#pragma unroll
        for (int m = 0; m < R / 2; ++m) rb.Dp[m] = Dc[m];
    }
    uint32_t c = c_first;
    const uint32_t peel_end = min(c_hi, ib + R + 1);
    for (; c < peel_end; ++c)
        column_step2<R, true>(rb, cols, base, c, ib, n, Q, margin, B, best);
    for (; c < c_hi; ++c)
        column_step2<R, false>(rb, cols, base, c, ib, n, Q, margin, B, best);
}

}  // namespace logo
