// Neighbour-list 2-opt search (LOGO_SEARCH_NEIGHBOUR).
//
// The candidate moves of a neighbour sweep are the ones that create an edge
// from a city to one of its K nearest cities: for tour position i (city
// t = route[i]) and each listed neighbour v of t at position p = pos[v],
// with (a, b) = (min(i, p), max(i, p)) and b >= a + 2,
//     pair (a, b):         d(a, b) + d(a-1, b-1) - e[a] - e[b]   (a >= 1)
//     pair (a+1, b+1):     d(a+1, b+1) + d(a, b) - e[a+1] - e[b+1]   (b+1 <= n-1)
// -- both exact pairs of the full sweep (delta(i, c) with 1 <= i,
// i + 2 <= c <= n - 1), evaluated with the same per-edge distance.  The
// sweep keeps the lowest packed (delta, i, c) key among the improving ones,
// so one sweep evaluates 2Kn pairs instead of (n-2)(n-3)/2.  A descent in
// this mode applies such moves until no candidate improves and then
// continues with full sweeps to a 2-opt local optimum of the whole pair
// set: the end point is a local optimum like the reference's, reached along
// another path (no counterpart in the reference; the classic neighbour-list
// restriction of 2-opt, with the candidate order fixed by the packed key).
#include <algorithm>
#include <atomic>
#include <climits>

#include "logo_device.cuh"
#include "logo_internal.h"

namespace logo {

namespace {

constexpr int kNbrThreads = 256, kNbrThreadsOr = 128;
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

// One thread per tour position i; its city's neighbours in batches of
// kNbrBatch, every load of a batch issued before any is used (indices
// clamped into range, so the loads of candidates that do not exist are
// harmless).  With OR the same loads also serve the Or-opt candidates in
// which the city at i is a segment end: as the first city of the segments
// starting at i (lengths 1-3) and as the last city of the segments [i-1, i+1)
// and [i-2, i+1) -- every Or-opt candidate of the neighbour search exactly
// once per list entry, the same set as walking each segment's two end lists.
template <bool OR, int NT>
__global__ void __launch_bounds__(NT)
    nbr_sweep_kernel(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                     const uint32_t* __restrict__ R0, const uint32_t* __restrict__ R1,
                     const uint32_t* __restrict__ pos, const uint32_t* __restrict__ nbr,
                     uint32_t K, uint32_t n, float M, DevState* st) {
    chain_wait();
    chain_release();
    __shared__ unsigned long long red[NT / 32];
    __shared__ unsigned long long red_or[OR ? kOrSlots : 1][NT / 32];
    if (*(volatile unsigned int*)&st->converged) return;  // the same in every thread
    const bool cur = *(volatile unsigned int*)&st->cur;
    const OrderedCity* Q = cur ? Q1 : Q0;
    const uint32_t* R = cur ? R1 : R0;
    uint64_t best = kNoMove;
    uint64_t bo[kOrSlots];
#pragma unroll
    for (int v = 0; v < kOrSlots; ++v) bo[v] = kNoMove;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const uint32_t city = min(R[i], n - 1);
        const OrderedCity qim = Q[i >= 1 ? i - 1 : 0], qi = Q[i], qip = Q[min(i + 1, n - 1)];
        // Or-opt: positions i-3 .. i+3 and the bases d(s-1, s+L) - e[s] - e[s+L]
        // of the segments (s, L) = (i, 1), (i, 2), (i, 3), (i-1, 2), (i-2, 3)
        OrderedCity qm3, qm2, qp2, qp3;
        int b1 = INT_MAX, b2 = INT_MAX, b3 = INT_MAX, c2 = INT_MAX, c3 = INT_MAX;
        if (OR) {
            qm3 = Q[i >= 3 ? i - 3 : 0];
            qm2 = Q[i >= 2 ? i - 2 : 0];
            qp2 = Q[min(i + 2, n - 1)];
            qp3 = Q[min(i + 3, n - 1)];
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
            for (uint32_t j = 0; j < kNbrBatch; ++j) p[j] = min(pos[min(p[j], n - 1)], n - 1);
            OrderedCity qpm[kNbrBatch], qp[kNbrBatch], qpp[kNbrBatch];
#pragma unroll
            for (uint32_t j = 0; j < kNbrBatch; ++j) {
                qpm[j] = Q[p[j] >= 1 ? p[j] - 1 : 0];
                qp[j] = Q[p[j]];
                qpp[j] = Q[min(p[j] + 1, n - 1)];
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
    best = warp_min_u64(best);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = best;
    if (OR) {
#pragma unroll
        for (int v = 0; v < kOrSlots; ++v) {
            const uint64_t m = warp_min_u64(bo[v]);
            if (lane == 0) red_or[v][warp] = m;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t m = red[0];
        for (int w = 1; w < NT / 32; ++w) m = red[w] < m ? red[w] : m;
        if (m != kNoMove) atomicMin(&st->best_key, (unsigned long long)m);
        if (OR) {
            for (int v = 0; v < kOrSlots; ++v) {
                uint64_t mv = red_or[v][0];
                for (int w = 1; w < NT / 32; ++w) mv = red_or[v][w] < mv ? red_or[v][w] : mv;
                if (mv != kNoMove) atomicMin(&st->or_key[v], (unsigned long long)mv);
            }
        }
        if (blockIdx.x == 0) st->nbr_sweeps += 1;
    }
}

// pos[route_cur[k]] = k for every position (after pos was not maintained).
__global__ void fill_pos_kernel(const uint32_t* __restrict__ R0, const uint32_t* __restrict__ R1,
                                uint32_t* __restrict__ pos, uint32_t n, const DevState* st) {
    const uint32_t* R = *(volatile const unsigned int*)&st->cur ? R1 : R0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        pos[min(R[k], n - 1)] = k;
}

}  // namespace

cudaError_t launch_nbr_sweep(const NbrLaunch& L, cudaStream_t s) {
    // the Or-opt variant holds more state per thread: smaller CTAs keep one
    // wave resident
    const int nt = L.oropt ? kNbrThreadsOr : kNbrThreads;
    const uint64_t blocks = ((uint64_t)L.n + nt - 1) / nt;
    unsigned grid = (unsigned)(blocks < 1 ? 1 : (blocks > 16384 ? 16384 : blocks));
    if (L.oropt) {
        // no more CTAs than are resident at once (the loop strides over the
        // rest): a second wave of a few CTAs would cost a whole CTA's time
        static std::atomic<unsigned> resident[64];
        int device = 0;
        cudaError_t e = cudaGetDevice(&device);
        if (e != cudaSuccess) return e;
        unsigned r = resident[(unsigned)device % 64].load(std::memory_order_relaxed);
        if (r == 0) {
            int sms = 0, per_sm = 0;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, nbr_sweep_kernel<true, kNbrThreadsOr>, kNbrThreadsOr, 0);
            if (e != cudaSuccess) return e;
            r = (unsigned)(per_sm > 0 ? per_sm : 1) * (unsigned)sms;
            resident[(unsigned)device % 64].store(r, std::memory_order_relaxed);
        }
        grid = grid < r ? grid : r;
    }
    if (L.oropt)
        return launch_chained(nbr_sweep_kernel<true, kNbrThreadsOr>, grid, kNbrThreadsOr, 0, s,
                              L.Q0, L.Q1, L.R0, L.R1, L.pos, L.nbr, L.K, L.n, L.margin, L.st);
    return launch_chained(nbr_sweep_kernel<false, kNbrThreads>, grid, kNbrThreads, 0, s, L.Q0,
                          L.Q1, L.R0, L.R1, L.pos, L.nbr, L.K, L.n, L.margin, L.st);
}

cudaError_t launch_fill_pos(const NbrLaunch& L, cudaStream_t s) {
    const unsigned grid = (unsigned)std::min<uint64_t>((L.n + 255) / 256, 4096);
    fill_pos_kernel<<<grid < 1 ? 1 : grid, 256, 0, s>>>(L.R0, L.R1, L.pos, L.n, L.st);
    return cudaGetLastError();
}

}  // namespace logo
