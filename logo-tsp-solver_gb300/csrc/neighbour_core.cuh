// Candidate evaluation of the neighbour-list search (LOGO_SEARCH_NEIGHBOUR,
// LOGO_SEARCH_NEIGHBOUR_OROPT), shared by the sweep kernel of neighbour.cu
// and the cooperative neighbour descent of coop.cu.  See neighbour.cu for
// the candidate set.
#pragma once
#include <climits>

#include "logo_device.cuh"

namespace logo {

// Loads of the tour (ordered cities, route, positions).  kLdPlain: the
// multi-kernel path, where the tour is read-only for the whole launch.
// kLdCoherent: the cooperative phase, where other SMs rewrite the tour
// between moves of one launch: coherent (ld.global.ca, never the read-only
// path), made current after each grid barrier by its acquire.  kLdL2: the
// same through L2 only.
constexpr int kLdPlain = 0, kLdL2 = 1, kLdCoherent = 2;
template <int LD>
__device__ __forceinline__ OrderedCity ld_city(const OrderedCity* p) {
    if (LD != kLdPlain) {
        const float4* q = reinterpret_cast<const float4*>(p);
        const float4 v = LD == kLdL2 ? __ldcg(q) : __ldca(q);
        OrderedCity o;
        o.x = v.x;
        o.y = v.y;
        o.e = v.z;
        o.pad = v.w;
        return o;
    }
    return *p;
}
template <int LD>
__device__ __forceinline__ uint32_t ld_u32(const uint32_t* p) {
    return LD == kLdPlain ? *p : (LD == kLdL2 ? __ldcg(p) : __ldca(p));
}

constexpr uint32_t kNbrBatch = 4;  // neighbours whose loads are issued together

// The two candidate pairs of position i (qim, qi, qip: positions i-1, i,
// i+1) with the city at position p (qpm, qp, qpp likewise), kept in best.
__device__ __forceinline__ void nbr_pairs(uint32_t i, uint32_t p, uint32_t n, OrderedCity qim,
                                          OrderedCity qi, OrderedCity qip, OrderedCity qpm,
                                          OrderedCity qp, OrderedCity qpp, uint64_t& best) {
    const bool ilo = i < p;
    const uint32_t a = ilo ? i : p, b = ilo ? p : i;
    if (b < a + 2) return;
    const OrderedCity qa = ilo ? qi : qp, qb = ilo ? qp : qi;
    const OrderedCity qam = ilo ? qim : qpm, qbm = ilo ? qpm : qim;
    const OrderedCity qap = ilo ? qip : qpp, qbp = ilo ? qpp : qip;
    const int D = exact_dist(qa.x, qa.y, qb.x, qb.y);
    if (a >= 1) {
        const int delta = D + exact_dist(qam.x, qam.y, qbm.x, qbm.y) - (int)qa.e - (int)qb.e;
        if (delta < 0) {
            const uint64_t key = pack_key(delta, a, b);
            best = key < best ? key : best;
        }
    }
    if (b + 1 <= n - 1) {
        const int delta = exact_dist(qap.x, qap.y, qbp.x, qbp.y) + D - (int)qap.e - (int)qbp.e;
        if (delta < 0) {
            const uint64_t key = pack_key(delta, a + 1, b + 1);
            best = key < best ? key : best;
        }
    }
}

// An Or-opt candidate of the segment [s, s+L) (first and last: its end
// cities) moved into the gap after old position p (qp, qp1: positions p and
// p+1); base = d(s-1, s+L) - e[s] - e[s+L], or INT_MAX where the segment
// does not exist.  Forward: new edges (p, s) and (s+L-1, p+1); reversed:
// (p, s+L-1) and (s, p+1).  The two new distances are first estimated with
// the MUFU square root: the exact delta is at least the estimate minus M
// (filter_margin: two approximate distances, three roundings of magnitudes
// up to four diagonals, as for a 2-opt pair), so an estimate >= M rules the
// candidate out and only the others are evaluated exactly.
template <int L, bool REV>
__device__ __forceinline__ void or_try(uint32_t s, uint32_t p, uint32_t n,
                                       const OrderedCity& first, const OrderedCity& last,
                                       int base, float M, const OrderedCity& qp,
                                       const OrderedCity& qp1, uint64_t* bo) {
    if (base == INT_MAX) return;
    if (!(p + 2 <= s || (p >= s + (uint32_t)L && p + 2 <= n))) return;
    const OrderedCity& u = REV ? last : first;
    const OrderedCity& w = REV ? first : last;
    const float v = (float)base + approx_dist(qp.x, qp.y, u.x, u.y) +
                    (approx_dist(w.x, w.y, qp1.x, qp1.y) - qp1.e);
    if (!(v < M)) return;
    const int delta = base + exact_dist(qp.x, qp.y, u.x, u.y) +
                      exact_dist(w.x, w.y, qp1.x, qp1.y) - (int)qp1.e;
    if (delta < 0) {
        constexpr int slot = L == 1 ? 0 : 2 * L - 3 + (REV ? 1 : 0);
        const uint64_t key = pack_key(delta, s, p);
        bo[slot] = key < bo[slot] ? key : bo[slot];
    }
}

// Every candidate of tour position i (its city's list: 2-opt pairs, and
// with OR the Or-opt moves in which the city at i is a segment end); the
// lowest 2-opt key goes to best and the lowest Or-opt key per variant to bo.
template <bool OR, int LD = kLdPlain>
__device__ __forceinline__ void nbr_position(uint32_t i, const OrderedCity* __restrict__ Q,
                                             const uint32_t* __restrict__ R,
                                             const uint32_t* __restrict__ pos,
                                             const uint32_t* __restrict__ nbr, uint32_t K,
                                             uint32_t n, float M, uint64_t& best,
                                             uint64_t* bo) {
    const uint32_t city = min(ld_u32<LD>(R + i), n - 1);
    const OrderedCity qim = ld_city<LD>(Q + (i >= 1 ? i - 1 : 0)), qi = ld_city<LD>(Q + i),
                      qip = ld_city<LD>(Q + min(i + 1, n - 1));
    // Or-opt: positions i-3 .. i+3 and the bases d(s-1, s+L) - e[s] - e[s+L]
    // of the segments (s, L) = (i, 1), (i, 2), (i, 3), (i-1, 2), (i-2, 3)
    OrderedCity qm3, qm2, qp2, qp3;
    int b1 = INT_MAX, b2 = INT_MAX, b3 = INT_MAX, c2 = INT_MAX, c3 = INT_MAX;
    if (OR) {
        qm3 = ld_city<LD>(Q + (i >= 3 ? i - 3 : 0));
        qm2 = ld_city<LD>(Q + (i >= 2 ? i - 2 : 0));
        qp2 = ld_city<LD>(Q + min(i + 2, n - 1));
        qp3 = ld_city<LD>(Q + min(i + 3, n - 1));
        if (i >= 1 && i + 1 <= n - 1)
            b1 = exact_dist(qim.x, qim.y, qip.x, qip.y) - (int)qi.e - (int)qip.e;
        if (i >= 1 && i + 2 <= n - 1)
            b2 = exact_dist(qim.x, qim.y, qp2.x, qp2.y) - (int)qi.e - (int)qp2.e;
        if (i >= 1 && i + 3 <= n - 1)
            b3 = exact_dist(qim.x, qim.y, qp3.x, qp3.y) - (int)qi.e - (int)qp3.e;
        if (i >= 2 && i + 1 <= n - 1)  // segment [i-1, i+1): s-1 = i-2, s+L = i+1
            c2 = exact_dist(qm2.x, qm2.y, qip.x, qip.y) - (int)qim.e - (int)qip.e;
        if (i >= 3 && i + 1 <= n - 1)  // segment [i-2, i+1): s-1 = i-3, s+L = i+1
            c3 = exact_dist(qm3.x, qm3.y, qip.x, qip.y) - (int)qm2.e - (int)qip.e;
    }
    const uint32_t* nb = nbr + (size_t)city * K;
    for (uint32_t k0 = 0; k0 < K; k0 += kNbrBatch) {
        uint32_t p[kNbrBatch];
#pragma unroll
        for (uint32_t j = 0; j < kNbrBatch; ++j) p[j] = nb[min(k0 + j, K - 1)];
#pragma unroll
        for (uint32_t j = 0; j < kNbrBatch; ++j) p[j] = min(ld_u32<LD>(pos + min(p[j], n - 1)), n - 1);
        OrderedCity qpm[kNbrBatch], qp[kNbrBatch], qpp[kNbrBatch];
#pragma unroll
        for (uint32_t j = 0; j < kNbrBatch; ++j) {
            qpm[j] = ld_city<LD>(Q + (p[j] >= 1 ? p[j] - 1 : 0));
            qp[j] = ld_city<LD>(Q + p[j]);
            qpp[j] = ld_city<LD>(Q + min(p[j] + 1, n - 1));
        }
#pragma unroll
        for (uint32_t j = 0; j < kNbrBatch; ++j) {
            if (k0 + j >= K) continue;
            nbr_pairs(i, p[j], n, qim, qi, qip, qpm[j], qp[j], qpp[j], best);
            if (!OR) continue;
            const uint32_t q = p[j];
            // the city at i first in the segments starting at i
            or_try<1, false>(i, q, n, qi, qi, b1, M, qp[j], qpp[j], bo);
            or_try<2, false>(i, q, n, qi, qip, b2, M, qp[j], qpp[j], bo);
            or_try<3, false>(i, q, n, qi, qp2, b3, M, qp[j], qpp[j], bo);
            if (q >= 1) {
                or_try<1, false>(i, q - 1, n, qi, qi, b1, M, qpm[j], qp[j], bo);
                or_try<2, true>(i, q - 1, n, qi, qip, b2, M, qpm[j], qp[j], bo);
                or_try<3, true>(i, q - 1, n, qi, qp2, b3, M, qpm[j], qp[j], bo);
            }
            // the city at i last in the segments [i-1, i+1) and [i-2, i+1)
            if (i >= 2) {
                or_try<2, true>(i - 1, q, n, qim, qi, c2, M, qp[j], qpp[j], bo);
                if (q >= 1) or_try<2, false>(i - 1, q - 1, n, qim, qi, c2, M, qpm[j], qp[j], bo);
            }
            if (i >= 3) {
                or_try<3, true>(i - 2, q, n, qm2, qi, c3, M, qp[j], qpp[j], bo);
                if (q >= 1) or_try<3, false>(i - 2, q - 1, n, qm2, qi, c3, M, qpm[j], qp[j], bo);
            }
        }
    }
}

}  // namespace logo
