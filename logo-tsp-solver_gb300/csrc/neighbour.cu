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

#include "logo_device.cuh"
#include "logo_internal.h"

namespace logo {

namespace {

constexpr int kNbrThreads = 256;
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

// One thread per tour position; its neighbours in batches of kNbrBatch,
// every load of a batch issued before any is used (indices clamped into
// range, so the loads of pairs that do not exist are harmless).
__global__ void __launch_bounds__(kNbrThreads)
    nbr_sweep_kernel(const OrderedCity* __restrict__ Q0, const OrderedCity* __restrict__ Q1,
                     const uint32_t* __restrict__ R0, const uint32_t* __restrict__ R1,
                     const uint32_t* __restrict__ pos, const uint32_t* __restrict__ nbr,
                     uint32_t K, uint32_t n, DevState* st) {
    chain_wait();
    chain_release();
    __shared__ unsigned long long red[kNbrThreads / 32];
    if (*(volatile unsigned int*)&st->converged) return;  // the same in every thread
    const bool cur = *(volatile unsigned int*)&st->cur;
    const OrderedCity* Q = cur ? Q1 : Q0;
    const uint32_t* R = cur ? R1 : R0;
    uint64_t best = kNoMove;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const uint32_t city = min(R[i], n - 1);
        const OrderedCity qim = Q[i >= 1 ? i - 1 : 0], qi = Q[i], qip = Q[min(i + 1, n - 1)];
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
            for (uint32_t j = 0; j < kNbrBatch; ++j)
                if (k0 + j < K) nbr_pairs(i, p[j], n, qim, qi, qip, qpm[j], qp[j], qpp[j], best);
        }
    }
    best = warp_min_u64(best);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t m = red[0];
        for (int w = 1; w < kNbrThreads / 32; ++w) m = red[w] < m ? red[w] : m;
        if (m != kNoMove) atomicMin(&st->best_key, (unsigned long long)m);
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
    const uint64_t blocks = ((uint64_t)L.n + kNbrThreads - 1) / kNbrThreads;
    const unsigned grid = (unsigned)(blocks < 1 ? 1 : (blocks > 8192 ? 8192 : blocks));
    return launch_chained(nbr_sweep_kernel, grid, kNbrThreads, 0, s, L.Q0, L.Q1, L.R0, L.R1,
                          L.pos, L.nbr, L.K, L.n, L.st);
}

cudaError_t launch_fill_pos(const NbrLaunch& L, cudaStream_t s) {
    const unsigned grid = (unsigned)std::min<uint64_t>((L.n + 255) / 256, 4096);
    fill_pos_kernel<<<grid < 1 ? 1 : grid, 256, 0, s>>>(L.R0, L.R1, L.pos, L.n, L.st);
    return cudaGetLastError();
}

}  // namespace logo
