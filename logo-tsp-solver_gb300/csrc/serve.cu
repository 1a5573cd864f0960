// Serving rounds: continuous batching of independent requests at the
// granularity of a bounded work quantum (sm_103a).
//
// Every admitted request owns a slot: its coordinates, current tour and best
// tour stay resident in a device arena between rounds, and a small state
// record (phase, counters, PRNG state, lengths) in ServeSlot.  A round kernel
// hands the active slots to CTAs through an atomic queue; a CTA loads its
// slot's tour into shared memory and advances the request's ILS -- the same
// descent / accept-or-revert / kick sequence as logo_ils and the batched
// solver (src/solvers/ILSGlobalSolverSequential.cpp:60-100) -- until it has
// spent `budget_pairs` pair evaluations (checked between sweeps) or the
// request is finished, then writes the state back.  Between rounds the host
// retires finished requests and admits new ones, so requests that arrive while
// others run join the next round and share the GPU with them.
//
// A slot's computation depends only on its own input, never on which other
// slots share a round, so a request's result is the same alone and in any mix.
#include <cstdint>

#include "cta_tour.cuh"
#include "logo_device.cuh"
#include "batch_internal.h"
#include "serve_internal.h"
#include "sweep_core.cuh"

namespace logo {

namespace {

template <int R, int NT, int TC>
__global__ void __launch_bounds__(NT) serve_round_kernel(ServeArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ CtaShared<NT> S;
    __shared__ CtaWindows W;
    OrderedCity* Q = reinterpret_cast<OrderedCity*>(smem_raw);
    uint32_t* route = reinterpret_cast<uint32_t*>(smem_raw + sizeof(OrderedCity) * A.max_n);
    uint32_t* bestr = route + A.max_n;

    for (;;) {
        if (threadIdx.x == 0) S.idx = atomicAdd(A.queue, 1u);
        __syncthreads();
        const uint32_t unit = S.idx;
        __syncthreads();
        if (unit >= A.nunits) break;
        const uint32_t slot = A.units[unit];
        ServeSlot st = A.slots[slot];
        if (st.phase == kServeDone) continue;
        const uint32_t n = st.n;
        const float2* xy = A.coords + st.off;
        uint32_t* rio = A.route + st.off;
        uint32_t* bio = A.best + st.off;

        // load the resident tour (and best tour) into shared memory
        for (uint32_t k = threadIdx.x; k < n; k += NT) {
            const uint32_t c = rio[k];
            route[k] = c;
            bestr[k] = (st.phase == kServeInit) ? c : bio[k];
            const float2 p = xy[c];
            OrderedCity o;
            o.x = p.x;
            o.y = p.y;
            o.e = 0.f;
            o.pad = 0.f;
            Q[k] = o;
        }
        if (threadIdx.x == 0) fill_tile_table<R, TC>(S, n);
        __syncthreads();
        recompute_edges<NT>(Q, n);
        __syncthreads();
        if (st.phase == kServeInit) {
            st.start_len = tour_length<NT>(S, Q, n);
            st.best_len = st.start_len;
            st.phase = kServeDescent;
        }
        const unsigned long long pairs = n >= 4 ? (unsigned long long)(n - 2) * (n - 3) / 2 : 0;
        const unsigned long long move_cap = 64ull * n * n + 1024;
        unsigned long long spent = 0;
        uint64_t rng = st.rng;
        while (st.phase != kServeDone && spent < A.budget_pairs) {
            if (st.phase == kServeDescent) {
                window_stats_cta<NT>(W, Q, n);
                __syncthreads();
                const unsigned long long key = sweep_boxed<R, NT, TC>(S, W, Q, n, st.margin);
                ++st.sweeps;
                spent += pairs + n;  // + n: a sweep of a tiny tour still costs work
                if (key == kNoMove) {
                    st.phase = kServeAccept;
                    continue;
                }
                const uint32_t p = key_i(key), q = key_j(key);
                if (!(p >= 1 && q < n && q >= p + 2)) {
                    st.status |= kErrBadKey;
                    st.phase = kServeDone;
                    break;
                }
                rotate_reverse<NT>(Q, route, n, p, q);
                ++st.moves;
                if (++st.descent_moves >= move_cap) {
                    st.status |= kErrMoveLimit;
                    st.phase = kServeDone;
                }
            } else {  // kServeAccept: keep if strictly shorter, else revert
                const unsigned long long len = tour_length<NT>(S, Q, n);
                if (len < st.best_len) {
                    st.best_len = len;
                    ++st.accepted;
                    for (uint32_t k = threadIdx.x; k < n; k += NT) bestr[k] = route[k];
                } else {
                    for (uint32_t k = threadIdx.x; k < n; k += NT) {
                        const uint32_t c = bestr[k];
                        route[k] = c;
                        const float2 p = xy[c];
                        Q[k].x = p.x;
                        Q[k].y = p.y;
                    }
                    __syncthreads();
                    recompute_edges<NT>(Q, n);
                }
                __syncthreads();
                if (st.kicks_done == st.kicks_total) {
                    st.phase = kServeDone;
                    break;
                }
                if (st.kick_kind == 1) {
                    uint32_t c0 = 1 + uniform_below(rng, n - 1);
                    uint32_t c1 = 1 + uniform_below(rng, n - 1);
                    uint32_t c2 = 1 + uniform_below(rng, n - 1);
                    uint32_t t;
                    if (c1 < c0) { t = c0; c0 = c1; c1 = t; }
                    if (c2 < c1) { t = c1; c1 = c2; c2 = t; }
                    if (c1 < c0) { t = c0; c0 = c1; c1 = t; }
                    double_bridge<NT>(Q, route, n, c0, c1, c2);
                } else {
                    uint32_t a = uniform_below(rng, n);
                    uint32_t b = uniform_below(rng, n);
                    if (b < a) { const uint32_t t = a; a = b; b = t; }
                    rotate_reverse<NT>(Q, route, n, a, b);
                }
                ++st.kicks_done;
                st.descent_moves = 0;
                st.phase = kServeDescent;
            }
        }
        st.rng = rng;
        // write the resident state back
        for (uint32_t k = threadIdx.x; k < n; k += NT) {
            rio[k] = route[k];
            bio[k] = bestr[k];
        }
        if (threadIdx.x == 0) A.slots[slot] = st;
        __syncthreads();
    }
}

}  // namespace

size_t serve_smem_bytes(uint32_t max_n) {
    return (size_t)max_n * (sizeof(OrderedCity) + 2 * sizeof(uint32_t));
}

// One compiled shape: R = 4 rows per thread, 256 threads, 128-column warp
// tiles (the fastest measured batched shape for n in [1024, 4096]).
constexpr int kServeR = 4, kServeNT = 256, kServeTC = 128;

cudaError_t launch_serve_round(const ServeArgs& A, int grid, cudaStream_t s, int* occupancy) {
    const size_t smem = serve_smem_bytes(A.max_n);
    auto kern = serve_round_kernel<kServeR, kServeNT, kServeTC>;
    if (occupancy) {
        // for the largest request: the attribute is shared by every server
        const size_t cap = serve_smem_bytes(kBatchMaxN);
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(cap > 48 * 1024 ? cap : 48 * 1024));
        if (e != cudaSuccess) return e;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy, kern, kServeNT, smem);
    }
    kern<<<grid, kServeNT, smem, s>>>(A);
    return cudaGetLastError();
}

}  // namespace logo
