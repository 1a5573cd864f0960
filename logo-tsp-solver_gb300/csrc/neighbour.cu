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
#include "neighbour_core.cuh"

namespace logo {

namespace {

constexpr int kNbrThreads = 256, kNbrThreadsOr = 128;

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
        nbr_position<OR>(i, Q, R, pos, nbr, K, n, M, best, bo);
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
