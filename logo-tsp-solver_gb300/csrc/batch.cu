// Batched persistent solver: many independent instances (n <= a few
// thousand) in one launch, each solved end to end -- descent, then ILS
// kicks with accept/revert -- by one CTA with the whole instance resident in
// shared memory (sm_103a).
//
// No reference counterpart: the reference solves one instance per process
// (or one per pthread, ILSGlobalSolverMT.cpp:86-195) and crosses the PCIe bus
// three times per move.  The per-instance algorithm is the reference's:
//   sweep     ≙ CPUSolver::optimizeStep loop order, per-edge nint
//               (src/solvers/cpuSolver.cpp:188-230) -- sweep_core.cuh
//   move      ≙ rotate + reverse (src/solvers/twoOptLocalSolver.cpp:41-48)
//   descent   ≙ TwoOptLocalSolver::optimize (twoOptLocalSolver.cpp:22-64)
//   ILS       ≙ ILSGlobalSolverSequential::optimize with a kick count
//               (src/solvers/ILSGlobalSolverSequential.cpp:60-100)
//   kick      ≙ ILSGlobalSolver::kick (ILSGlobalSolver.cpp:37-48) or the
//               double bridge
// so every instance ends with the same tour as the single-instance path.
//
// Scheduling: a global atomic work queue over instances sorted by descending
// n (longest first); each CTA pops the next instance when it finishes one.
// In shared memory the tour is permuted in place: a move
// new = old[i..c) ++ rev(old[0..i)) ++ rev(old[c..n)) is the three reversals
// rev[i,c) + rev[c,n) (disjoint, one phase), then rev[0,c).
#include <cstdint>

#include "batch_internal.h"
#include "logo_device.cuh"
#include "sweep_core.cuh"

namespace logo {

namespace {

template <int NT>
struct BatchShared {
    unsigned long long wbest[NT / 32];
    unsigned long long wsum[NT / 32];
    unsigned long long key;
    unsigned long long sum;
    unsigned int idx;
    unsigned int p, q, r;  // permutation parameters broadcast by thread 0
    unsigned int tiles_before[72];
};

__device__ __forceinline__ void swap_q(OrderedCity* Q, uint32_t* route, uint32_t a,
                                       uint32_t b) {
    const float4 qa = *reinterpret_cast<float4*>(Q + a);
    const float4 qb = *reinterpret_cast<float4*>(Q + b);
    *reinterpret_cast<float4*>(Q + a) = qb;
    *reinterpret_cast<float4*>(Q + b) = qa;
    const uint32_t ra = route[a];
    route[a] = route[b];
    route[b] = ra;
}

// Reverses [a0, a1) and [b0, b1) (disjoint) in one pass.
template <int NT>
__device__ __forceinline__ void reverse2(OrderedCity* Q, uint32_t* route, uint32_t a0,
                                         uint32_t a1, uint32_t b0, uint32_t b1) {
    const uint32_t ha = (a1 - a0) / 2, hb = (b1 - b0) / 2;
    for (uint32_t t = threadIdx.x; t < ha + hb; t += NT) {
        if (t < ha)
            swap_q(Q, route, a0 + t, a1 - 1 - t);
        else
            swap_q(Q, route, b0 + (t - ha), b1 - 1 - (t - ha));
    }
}

template <int NT>
__device__ __forceinline__ void recompute_edges(OrderedCity* Q, uint32_t n) {
    for (uint32_t k = threadIdx.x; k < n; k += NT) {
        const OrderedCity a = Q[k];
        const OrderedCity b = Q[k == 0 ? n - 1 : k - 1];
        Q[k].e = (float)exact_dist(b.x, b.y, a.x, a.y);
    }
}

// new = old[p..q) ++ rev(old[0..p)) ++ rev(old[q..n)), p <= q.
template <int NT>
__device__ __forceinline__ void rotate_reverse(OrderedCity* Q, uint32_t* route, uint32_t n,
                                               uint32_t p, uint32_t q) {
    reverse2<NT>(Q, route, p, q, q, n);
    __syncthreads();
    reverse2<NT>(Q, route, 0, q, 0, 0);
    __syncthreads();
    recompute_edges<NT>(Q, n);
    __syncthreads();
}

// new = old[0,p1) old[p2,p3) old[p1,p2) old[p3,n).
template <int NT>
__device__ __forceinline__ void double_bridge(OrderedCity* Q, uint32_t* route, uint32_t n,
                                              uint32_t p1, uint32_t p2, uint32_t p3) {
    reverse2<NT>(Q, route, p1, p3, 0, 0);
    __syncthreads();
    const uint32_t m = p1 + (p3 - p2);
    reverse2<NT>(Q, route, p1, m, m, p3);
    __syncthreads();
    recompute_edges<NT>(Q, n);
    __syncthreads();
}

template <int NT>
__device__ __forceinline__ unsigned long long block_sum(BatchShared<NT>& S,
                                                        unsigned long long v) {
    v = warp_sum_u64(v);
    if ((threadIdx.x & 31) == 0) S.wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; ++w) t += S.wsum[w];
        S.sum = t;
    }
    __syncthreads();
    const unsigned long long r = S.sum;
    __syncthreads();
    return r;
}

template <int NT>
__device__ __forceinline__ unsigned long long tour_length(BatchShared<NT>& S,
                                                          const OrderedCity* Q, uint32_t n) {
    unsigned long long s = 0;
    for (uint32_t k = threadIdx.x; k < n; k += NT) s += (unsigned long long)Q[k].e;
    return block_sum<NT>(S, s);
}

// One best-improvement sweep of the resident instance; returns the packed
// key of the best move (kNoMove if none).  Work: warp tiles of 32R rows x TC
// columns dealt round-robin to the warps.
template <int R, int NT, int TC>
__device__ __forceinline__ unsigned long long sweep(BatchShared<NT>& S, const OrderedCity* Q,
                                                    uint32_t n, float margin) {
    constexpr int NW = NT / 32;
    constexpr uint32_t RT = 32 * R;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t best = kNoMove;
    if (n >= 5) {
        const uint32_t nrb = (n - 3 + RT - 1) / RT;  // row blocks over rows 1..n-3
        const uint32_t total = S.tiles_before[nrb];
        uint32_t rbk = 0;
        for (uint32_t t = warp; t < total; t += NW) {
            while (S.tiles_before[rbk + 1] <= t) ++rbk;
            const uint32_t row0 = 1 + rbk * RT;
            const uint32_t col0 = row0 + 2 + (t - S.tiles_before[rbk]) * TC;
            const uint32_t col1 = min(col0 + TC, n);
            const uint32_t ib = row0 + lane * R;
            int B = -1;
            RowBlock<R> rb;
            load_rows<R>(rb, Q, ib, n);
            refresh_thresholds<R>(rb, Q, ib, n, B, margin);
            walk_columns<R>(rb, Q, 0, col0, col1, ib, n, Q, margin, B, best);
        }
    }
    best = warp_min_u64(best);
    if (lane == 0) S.wbest[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = S.wbest[0];
#pragma unroll
        for (int w = 1; w < NW; ++w) m = S.wbest[w] < m ? S.wbest[w] : m;
        S.key = m;
    }
    __syncthreads();
    const unsigned long long k = S.key;
    __syncthreads();
    return k;
}

template <int R, int NT, int TC>
__global__ void __launch_bounds__(NT)
    batch_kernel(BatchArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ BatchShared<NT> S;
    OrderedCity* Q = reinterpret_cast<OrderedCity*>(smem_raw);
    uint32_t* route = reinterpret_cast<uint32_t*>(smem_raw + sizeof(OrderedCity) * A.max_n);
    uint32_t* bestr = route + A.max_n;
    constexpr uint32_t RT = 32 * R;

    for (;;) {
        if (threadIdx.x == 0) S.idx = atomicAdd(A.queue, 1u);
        __syncthreads();
        const uint32_t slot = S.idx;
        __syncthreads();
        if (slot >= A.count) break;
        const uint32_t id = A.order[slot];
        const BatchInstance I = A.inst[id];
        const uint32_t n = I.n;
        const float2* xy = A.coords + I.off;
        uint32_t* rio = A.routes + I.off;

        // load the start tour, its ordered coordinates and edge lengths
        for (uint32_t k = threadIdx.x; k < n; k += NT) {
            const uint32_t c = rio[k];
            const float2 p = xy[c];
            route[k] = c;
            bestr[k] = c;
            OrderedCity o;
            o.x = p.x;
            o.y = p.y;
            o.e = 0.f;
            o.pad = 0.f;
            Q[k] = o;
        }
        if (threadIdx.x == 0) {
            // tiles per row block of the pair triangle (rows 1..n-3)
            uint32_t acc = 0, rbk = 0;
            S.tiles_before[0] = 0;
            if (n >= 5) {
                for (uint32_t row0 = 1; row0 + 3 <= n; row0 += RT, ++rbk) {
                    acc += (n - row0 - 2 + TC - 1) / TC;
                    S.tiles_before[rbk + 1] = acc;
                }
            }
        }
        __syncthreads();
        recompute_edges<NT>(Q, n);
        __syncthreads();
        const unsigned long long start_len = tour_length<NT>(S, Q, n);
        unsigned long long best_len = start_len;
        unsigned long long moves = 0, sweeps = 0;
        uint32_t accepted = 0, status = 0;
        uint64_t rng = I.seed;
        const unsigned long long move_cap = 64ull * n * n + 1024;

        for (uint32_t it = 0;; ++it) {
            // descent
            unsigned long long dm = 0;
            for (;;) {
                const unsigned long long key = sweep<R, NT, TC>(S, Q, n, I.margin);
                ++sweeps;
                if (key == kNoMove) break;
                const uint32_t p = key_i(key), q = key_j(key);
                if (!(p >= 1 && q < n && q >= p + 2)) {
                    status |= kErrBadKey;
                    break;
                }
                rotate_reverse<NT>(Q, route, n, p, q);
                ++moves;
                if (++dm >= move_cap) {
                    status |= kErrMoveLimit;
                    break;
                }
            }
            if (status) break;
            // accept (strictly shorter) or revert to the best tour
            const unsigned long long len = tour_length<NT>(S, Q, n);
            if (len < best_len) {
                best_len = len;
                ++accepted;
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
            if (it == A.kicks) break;
            // kick: every thread draws the same numbers from the same state
            if (A.kick_kind == 1) {
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
        }
        for (uint32_t k = threadIdx.x; k < n; k += NT) rio[k] = bestr[k];
        if (threadIdx.x == 0) {
            BatchResult r;
            r.start_length = start_len;
            r.best_length = best_len;
            r.moves = moves;
            r.sweeps = sweeps;
            r.kicks = status ? 0u : A.kicks;
            r.accepted = accepted;
            r.status = status;
            r.pad = 0;
            A.results[id] = r;
        }
        __syncthreads();
    }
}

}  // namespace

size_t batch_smem_bytes(uint32_t max_n) {
    return (size_t)max_n * (sizeof(OrderedCity) + 2 * sizeof(uint32_t));
}

template <int R, int NT, int TC>
static cudaError_t launch_batch_t(const BatchArgs& A, int grid, cudaStream_t s,
                                  int* occupancy) {
    const size_t smem = batch_smem_bytes(A.max_n);
    if (occupancy) {
        // the attribute is set here, outside any stream capture
        cudaError_t e = cudaFuncSetAttribute(batch_kernel<R, NT, TC>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(smem > 48 * 1024 ? smem : 48 * 1024));
        if (e != cudaSuccess) return e;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy, batch_kernel<R, NT, TC>,
                                                             NT, smem);
    }
    batch_kernel<R, NT, TC><<<grid, NT, smem, s>>>(A);
    return cudaGetLastError();
}

#define LOGO_BATCH_SHAPES(X) \
    X(2, 128, 64)            \
    X(2, 256, 64)            \
    X(4, 128, 64)            \
    X(4, 256, 64)            \
    X(4, 256, 128)           \
    X(4, 512, 128)           \
    X(8, 256, 128)

cudaError_t launch_batch(const BatchArgs& A, const BatchShape& sh, int grid, cudaStream_t s,
                         int* occupancy) {
#define X(r, nt, tc) \
    if (sh.R == r && sh.NT == nt && sh.TC == tc) return launch_batch_t<r, nt, tc>(A, grid, s, occupancy);
    LOGO_BATCH_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

int batch_shapes(BatchShape* out, int cap) {
    int k = 0;
#define X(r, nt, tc)                              \
    if (k < cap && out) out[k] = BatchShape{r, nt, tc}; \
    ++k;
    LOGO_BATCH_SHAPES(X)
#undef X
    return k;
}

}  // namespace logo
