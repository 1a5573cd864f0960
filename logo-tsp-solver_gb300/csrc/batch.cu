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
#include "cta_tour.cuh"
#include "sweep_core.cuh"

namespace logo {

static_assert((kBatchMaxN - 3 + kWin7 - 1) / kWin7 <= kCtaWindows,
              "the CTA sweep's window statistics cover the largest instance");

namespace {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned int* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Multi-start sharing (ILSGlobalSolverMT.cpp:86-195 with comm = 1): offers
// this replica's best tour to its group if it beats the group's best.  The
// lock is only tried, never waited for; a replica that finds it taken offers
// again after its next descent.
template <int NT>
__device__ void publish_best(SharedBest* g, uint32_t* tours, const uint32_t* bestr, uint32_t n,
                             unsigned long long best_len, unsigned int* flag) {
    if (threadIdx.x == 0) {
        unsigned int f = 0;
        if (best_len < *(volatile unsigned long long*)&g->best_len &&
            atomicCAS(&g->lock, 0u, 1u) == 0u) {
            if (best_len < *(volatile unsigned long long*)&g->best_len) {
                atomicAdd(&g->seq, 1u);  // odd: rewriting
                __threadfence();
                f = 1;
            } else {
                atomicExch(&g->lock, 0u);
            }
        }
        *flag = f;
    }
    __syncthreads();
    if (*flag) {
        uint32_t* t = tours + g->off;
        for (uint32_t k = threadIdx.x; k < n; k += NT) t[k] = bestr[k];
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            *(volatile unsigned long long*)&g->best_len = best_len;
            __threadfence();
            atomicAdd(&g->seq, 1u);  // even: consistent
            atomicExch(&g->lock, 0u);
        }
    }
    __syncthreads();
}

// Loads the group's best tour into route / Q (coordinates; the caller
// recomputes edges) when one is published that is no longer than this
// replica's best; false (route / Q possibly overwritten) when there is none
// or it changed while being read.
template <int NT>
__device__ bool adopt_best(SharedBest* g, const uint32_t* tours, uint32_t* route,
                           OrderedCity* Q, const float2* xy, uint32_t n,
                           unsigned long long best_len, unsigned int* flag, unsigned int* s1) {
    if (threadIdx.x == 0) {
        const unsigned int q = ld_acquire_u32(&g->seq);
        const unsigned long long gl = *(volatile unsigned long long*)&g->best_len;
        *s1 = q;
        *flag = !(q & 1u) && gl != ~0ull && gl <= best_len;
    }
    __syncthreads();
    if (!*flag) {
        __syncthreads();
        return false;
    }
    const uint32_t* t = tours + g->off;
    for (uint32_t k = threadIdx.x; k < n; k += NT) {
        const uint32_t c = __ldcg(t + k);
        route[k] = c < n ? c : 0u;
        const float2 p = xy[route[k]];
        Q[k].x = p.x;
        Q[k].y = p.y;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        *flag = ld_acquire_u32(&g->seq) == *s1;
    }
    __syncthreads();
    const bool ok = *flag;
    __syncthreads();
    return ok;
}

// Nearest-neighbour start tour of one instance, built by the CTA (the host
// logo_nn_tour, itself initRoute_KD_NN of src/utils/kdtree_utils.c:279-301):
// from city 0's point, repeatedly the nearest unvisited city by the double
// distance sqrt(dx*dx + dy*dy) (no contraction, as the host computes it), ties
// to the lowest id.  Each step screens the unvisited cities with the binary32
// squared distance, whose relative error is below 2.5e-7, so every city whose
// double distance can be the minimum has a float value within a factor
// 1 + 1e-6 of the float minimum; only those are evaluated in double.
template <int NT>
__device__ void nn_tour_cta(const float2* xy, uint32_t n, uint32_t* route, uint32_t* visited) {
    __shared__ float red_f[NT / 32];
    __shared__ double red_d[NT / 32];
    __shared__ uint32_t red_i[NT / 32];
    __shared__ uint32_t pick;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t k = threadIdx.x; k < n; k += NT) visited[k] = 0;
    __syncthreads();
    float px = xy[0].x, py = xy[0].y;
    for (uint32_t step = 0; step < n; ++step) {
        float m = INFINITY;
        for (uint32_t j = threadIdx.x; j < n; j += NT) {
            if (visited[j]) continue;
            const float dx = __fsub_rn(px, xy[j].x), dy = __fsub_rn(py, xy[j].y);
            m = fminf(m, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
        }
        for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) red_f[warp] = m;
        __syncthreads();
        m = red_f[0];
#pragma unroll
        for (int w = 1; w < NT / 32; ++w) m = fminf(m, red_f[w]);
        const float thr = m * (1.0f + 1e-6f) + 1e-30f;
        double bd = INFINITY;
        uint32_t bi = 0xFFFFFFFFu;
        for (uint32_t j = threadIdx.x; j < n; j += NT) {
            if (visited[j]) continue;
            const float2 q = xy[j];
            const float dx = __fsub_rn(px, q.x), dy = __fsub_rn(py, q.y);
            if (__fmaf_rn(dy, dy, __fmul_rn(dx, dx)) > thr) continue;
            const double ex = __dsub_rn((double)px, (double)q.x);
            const double ey = __dsub_rn((double)py, (double)q.y);
            const double d = __dsqrt_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)));
            if (d < bd || (d == bd && j < bi)) {
                bd = d;
                bi = j;
            }
        }
        for (int o = 16; o; o >>= 1) {
            const double od = __shfl_xor_sync(0xffffffffu, bd, o);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (od < bd || (od == bd && oi < bi)) {
                bd = od;
                bi = oi;
            }
        }
        if (lane == 0) {
            red_d[warp] = bd;
            red_i[warp] = bi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double d = red_d[0];
            uint32_t i = red_i[0];
            for (int w = 1; w < NT / 32; ++w)
                if (red_d[w] < d || (red_d[w] == d && red_i[w] < i)) {
                    d = red_d[w];
                    i = red_i[w];
                }
            pick = i < n ? i : 0u;
            route[step] = pick;
            visited[pick] = 1;
        }
        __syncthreads();
        px = xy[pick].x;
        py = xy[pick].y;
    }
}

// ---- multiple-fragment start tour, built by the CTA --------------------------
// The same steps as the host logo_mf_tour (csrc/construct.cpp), itself the
// steps of multipleFragment_KD (src/utils/kdtree_utils.c:56-242): every city
// links to its nearest other city; a priority queue of (nint distance to the
// link, city) is popped shortest first; a city of degree 2 is dropped, a
// link that is no longer usable (degree 2, or the far end of the city's own
// fragment) is looked up again among the cities of degree < 2 and the city
// re-queued; otherwise the two fragments are joined.  The host queue is
// std::priority_queue ordered by distance alone, so cities of equal distance
// leave it in the order of its sift steps; one thread replays those steps
// exactly (the standard binary heap: push sifts the new element up from the
// end; pop moves the hole from the root down to a leaf along the child that
// comes first, then sifts the former last element up from there), and the
// CTA answers the nearest-city queries as nn_tour_cta does (binary32 screen,
// double decision, lowest id on ties).  State in shared memory: the heap
// (8n bytes), 16-bit links and fragment ends, 8-bit degrees (together 13n
// bytes), 16-bit neighbours in join order (4n bytes); n <= 4096.  A kernel
// of its own (mf_start_kernel) builds every instance's tour before the
// batched solve, which then loads them as given tours.
struct MfFrag {
    int d;
    uint32_t id;
};

// a comes after b in the host's queue (its top is the shortest distance)
__device__ __forceinline__ bool mf_after(const MfFrag& a, const MfFrag& b) { return a.d > b.d; }

__device__ void mf_sift_up(MfFrag* H, int hole, int top, MfFrag v) {
    int parent = (hole - 1) / 2;
    while (hole > top && mf_after(H[parent], v)) {
        H[hole] = H[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    H[hole] = v;
}

__device__ void mf_push(MfFrag* H, int& len, MfFrag v) {
    mf_sift_up(H, len, 0, v);
    ++len;
}

__device__ void mf_pop(MfFrag* H, int& len) {
    const int nl = len - 1;
    const MfFrag v = H[nl];
    int hole = 0, child = 0;
    while (child < (nl - 1) / 2) {
        child = 2 * (child + 1);
        if (mf_after(H[child], H[child - 1])) --child;
        H[hole] = H[child];
        hole = child;
    }
    if ((nl & 1) == 0 && child == (nl - 2) / 2) {
        child = 2 * (child + 1);
        H[hole] = H[child - 1];
        hole = child - 1;
    }
    mf_sift_up(H, hole, 0, v);
    len = nl;
}

__device__ __forceinline__ double mf_ddist(float2 a, float2 b) {
    const double ex = __dsub_rn((double)a.x, (double)b.x);
    const double ey = __dsub_rn((double)a.y, (double)b.y);
    return __dsqrt_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)));
}

// One thread's nearest other city to city i among all cities (the initial
// links): binary32 squared distances screen, double decides, lowest id wins.
__device__ uint32_t mf_nearest_all(const float2* xy, uint32_t n, uint32_t i) {
    const float2 p = xy[i];
    float m = INFINITY;
    for (uint32_t j = 0; j < n; ++j) {
        if (j == i) continue;
        const float2 q = xy[j];
        const float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y);
        m = fminf(m, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    }
    const float thr = m * (1.0f + 1e-6f) + 1e-30f;
    double bd = INFINITY;
    uint32_t bi = i;
    for (uint32_t j = 0; j < n; ++j) {
        if (j == i) continue;
        const float2 q = xy[j];
        const float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y);
        if (__fmaf_rn(dy, dy, __fmul_rn(dx, dx)) > thr) continue;
        const double d = mf_ddist(p, q);
        if (d < bd) {  // j ascending: equal distances keep the lower id
            bd = d;
            bi = j;
        }
    }
    return bi;
}

// The CTA's nearest city to city x among those of degree < 2, other than x
// and skip; n (none) if there is no such city.  Every thread returns it.
template <int NT>
__device__ uint32_t mf_nearest_cta(const float2* xy, uint32_t n, uint32_t x, uint32_t skip,
                                   const uint8_t* degree) {
    __shared__ float red_f[NT / 32];
    __shared__ double red_d[NT / 32];
    __shared__ uint32_t red_i[NT / 32];
    __shared__ uint32_t pick;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float2 p = xy[x];
    float m = INFINITY;
    for (uint32_t j = threadIdx.x; j < n; j += NT) {
        if (j == x || j == skip || degree[j] >= 2) continue;
        const float2 q = xy[j];
        const float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y);
        m = fminf(m, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    }
    for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) red_f[warp] = m;
    __syncthreads();
    m = red_f[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) m = fminf(m, red_f[w]);
    const float thr = m * (1.0f + 1e-6f) + 1e-30f;
    double bd = INFINITY;
    uint32_t bi = 0xFFFFFFFFu;
    for (uint32_t j = threadIdx.x; j < n; j += NT) {
        if (j == x || j == skip || degree[j] >= 2) continue;
        const float2 q = xy[j];
        const float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y);
        if (__fmaf_rn(dy, dy, __fmul_rn(dx, dx)) > thr) continue;
        const double d = mf_ddist(p, q);
        if (d < bd || (d == bd && j < bi)) {
            bd = d;
            bi = j;
        }
    }
    for (int o = 16; o; o >>= 1) {
        const double od = __shfl_xor_sync(0xffffffffu, bd, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (od < bd || (od == bd && oi < bi)) {
            bd = od;
            bi = oi;
        }
    }
    if (lane == 0) {
        red_d[warp] = bd;
        red_i[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double d = red_d[0];
        uint32_t i = red_i[0];
        for (int w = 1; w < NT / 32; ++w)
            if (red_d[w] < d || (red_d[w] == d && red_i[w] < i)) {
                d = red_d[w];
                i = red_i[w];
            }
        pick = i < n ? i : n;
    }
    __syncthreads();
    const uint32_t r = pick;
    __syncthreads();
    return r;
}

template <int NT>
__device__ void mf_tour_cta(const float2* xy, uint32_t n, uint32_t* route, unsigned char* qbuf,
                            uint32_t* bbuf) {
    __shared__ int ctl;
    __shared__ uint32_t cx, cy, cskip;
    __shared__ int hlen;
    __shared__ bool failed;
    if (n <= 2) {  // as the host: nothing to join
        for (uint32_t k = threadIdx.x; k < n; k += NT) route[k] = k;
        __syncthreads();
        return;
    }
    MfFrag* H = reinterpret_cast<MfFrag*>(qbuf);
    uint16_t* link = reinterpret_cast<uint16_t*>(qbuf + 8 * (size_t)n);
    uint16_t* tail = link + n;
    uint8_t* degree = reinterpret_cast<uint8_t*>(qbuf + 12 * (size_t)n);
    int16_t* first = reinterpret_cast<int16_t*>(bbuf);
    int16_t* second = first + n;
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        tail[i] = (uint16_t)i;
        degree[i] = 0;
        first[i] = -1;
        second[i] = -1;
        link[i] = (uint16_t)mf_nearest_all(xy, n, i);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int len = 0;
        for (uint32_t i = 0; i < n; ++i) {
            const float2 a = xy[i], b = xy[link[i]];
            mf_push(H, len, MfFrag{exact_dist(a.x, a.y, b.x, b.y), i});
        }
        hlen = len;
        failed = false;
    }
    __syncthreads();
    // Between two joins a city is looked up again at most once (its new link
    // stays valid until the next join), so n * n bounds the look-ups of a
    // valid run; the count only guards the loop against a broken state.
    uint32_t requeries = 0;
    const uint32_t max_requeries = n * n + 64u;
    for (uint32_t e = 0; e + 1 < n && !failed; ++e) {
        for (;;) {
            if (threadIdx.x == 0) {
                int len = hlen;
                while (len > 0 && degree[H[0].id] == 2) mf_pop(H, len);
                hlen = len;
                if (len == 0) {
                    failed = true;
                    ctl = 0;
                } else {
                    const uint32_t x = H[0].id, y = link[x];
                    cx = x;
                    if (degree[y] < 2 && y != tail[x]) {
                        ctl = 0;
                        cy = y;
                    } else {
                        ctl = 1;
                        cskip = degree[x] ? tail[x] : x;
                    }
                }
            }
            __syncthreads();
            if (ctl == 0) break;
            if (++requeries > max_requeries) {  // the same in every thread
                if (threadIdx.x == 0) failed = true;
                __syncthreads();
                break;
            }
            const uint32_t nx = mf_nearest_cta<NT>(xy, n, cx, cskip, degree);
            if (threadIdx.x == 0) {
                if (nx >= n) {
                    failed = true;
                } else {
                    const uint32_t x = cx;
                    link[x] = (uint16_t)nx;
                    int len = hlen;
                    mf_pop(H, len);
                    const float2 a = xy[x], b = xy[nx];
                    mf_push(H, len, MfFrag{exact_dist(a.x, a.y, b.x, b.y), x});
                    hlen = len;
                }
            }
            __syncthreads();
            if (failed) break;
        }
        if (failed) break;
        if (threadIdx.x == 0) {
            const uint32_t x = cx, y = cy;
            const uint32_t vs[2] = {x, y};
            for (int t = 0; t < 2; ++t) {
                const uint32_t v = vs[t], w = t == 0 ? y : x;
                if (degree[v] == 0)
                    first[v] = (int16_t)w;
                else
                    second[v] = (int16_t)w;
                degree[v] = (uint8_t)(degree[v] + 1);
            }
            const uint32_t tx = tail[x];
            tail[tx] = tail[y];
            tail[tail[y]] = (uint16_t)tx;
        }
        __syncthreads();
    }
    // list the path from city 0: the part through first[0] reversed, 0, then
    // the part through second[0]
    if (threadIdx.x == 0 && !failed) {
        uint32_t len_before = 0;
        int from = 0, at = first[0];
        while (at >= 0 && len_before < n) {
            ++len_before;
            const int nx = first[at] == from ? second[at] : first[at];
            from = at;
            at = nx;
        }
        uint32_t k = len_before, count = 0;
        from = 0;
        at = first[0];
        while (at >= 0 && k > 0) {
            route[--k] = (uint32_t)at;
            ++count;
            const int nx = first[at] == from ? second[at] : first[at];
            from = at;
            at = nx;
        }
        k = len_before;
        if (k < n) route[k++] = 0;
        from = 0;
        at = second[0];
        while (at >= 0 && k < n) {
            route[k++] = (uint32_t)at;
            const int nx = first[at] == from ? second[at] : first[at];
            from = at;
            at = nx;
        }
        if (k != n || count != len_before) failed = true;
    }
    __syncthreads();
    if (failed)  // not reached for valid input; the tour stays a permutation
        for (uint32_t k = threadIdx.x; k < n; k += NT) route[k] = k;
    __syncthreads();
}

constexpr int kMfThreads = 256;

__global__ void __launch_bounds__(kMfThreads)
    mf_start_kernel(const float2* __restrict__ coords, uint32_t* __restrict__ routes,
                    const BatchInstance* __restrict__ inst, const uint32_t* __restrict__ order,
                    uint32_t count, uint32_t max_n) {
    extern __shared__ __align__(16) unsigned char mf_smem[];
    unsigned char* qbuf = mf_smem;
    uint32_t* bbuf = reinterpret_cast<uint32_t*>(mf_smem + ((13 * (size_t)max_n + 15) & ~(size_t)15));
    for (uint32_t k = blockIdx.x; k < count; k += gridDim.x) {
        const BatchInstance I = inst[order[k]];
        mf_tour_cta<kMfThreads>(coords + I.off, I.n, routes + I.off, qbuf, bbuf);
    }
}

size_t mf_smem_bytes(uint32_t max_n) {
    return ((13 * (size_t)max_n + 15) & ~(size_t)15) + 4 * (size_t)max_n;
}

// A start tour of one instance (logo_start_tour on a single-instance
// context): one CTA runs the batched launch's device builders (route
// written to global memory).
__global__ void __launch_bounds__(kMfThreads)
    start_tour_kernel(const float2* __restrict__ xy, uint32_t n, int kind, uint32_t* route) {
    extern __shared__ __align__(16) unsigned char st_smem[];
    if (kind == kStartNN) {
        nn_tour_cta<kMfThreads>(xy, n, route, reinterpret_cast<uint32_t*>(st_smem));
    } else {
        uint32_t* bbuf =
            reinterpret_cast<uint32_t*>(st_smem + ((13 * (size_t)n + 15) & ~(size_t)15));
        mf_tour_cta<kMfThreads>(xy, n, route, st_smem, bbuf);
    }
}

template <int R, int NT, int TC>
__global__ void __launch_bounds__(NT)
    batch_kernel(BatchArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ CtaShared<NT> S;
    __shared__ CtaWindows W;
    __shared__ unsigned int share_flag, share_seq;
    OrderedCity* Q = reinterpret_cast<OrderedCity*>(smem_raw);
    uint32_t* route = reinterpret_cast<uint32_t*>(smem_raw + sizeof(OrderedCity) * A.max_n);
    uint32_t* bestr = route + A.max_n;

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

        // load (or build) the start tour, its ordered coordinates and edge lengths
        if (A.start == kStartNN) nn_tour_cta<NT>(xy, n, route, bestr);
        for (uint32_t k = threadIdx.x; k < n; k += NT) {
            const uint32_t c = A.start == kStartNN ? route[k] : rio[k];
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
        if (threadIdx.x == 0) fill_tile_table<R, TC>(S, n);
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
                window_stats_cta<NT>(W, Q, n);
                __syncthreads();
                const unsigned long long key = sweep_boxed<R, NT, TC>(S, W, Q, n, I.margin);
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
            // accept (strictly shorter) or go back: to the replica's own best
            // tour, or in a multi-start group to the group's best
            const unsigned long long len = tour_length<NT>(S, Q, n);
            SharedBest* grp = I.group != kNoGroup ? A.shared + I.group : nullptr;
            if (len < best_len) {
                best_len = len;
                ++accepted;
                for (uint32_t k = threadIdx.x; k < n; k += NT) bestr[k] = route[k];
                __syncthreads();
            } else {
                const bool adopted = grp && adopt_best<NT>(grp, A.shared_tours, route, Q, xy, n,
                                                           best_len, &share_flag, &share_seq);
                if (!adopted) {
                    for (uint32_t k = threadIdx.x; k < n; k += NT) {
                        const uint32_t c = bestr[k];
                        route[k] = c;
                        const float2 p = xy[c];
                        Q[k].x = p.x;
                        Q[k].y = p.y;
                    }
                }
                __syncthreads();
                recompute_edges<NT>(Q, n);
            }
            __syncthreads();
            if (grp) publish_best<NT>(grp, A.shared_tours, bestr, n, best_len, &share_flag);
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
        // the attribute is set here, outside any stream capture, and for the
        // largest instance (it is shared by every batch object in the process)
        const size_t cap = batch_smem_bytes(kBatchMaxN);
        cudaError_t e = cudaFuncSetAttribute(batch_kernel<R, NT, TC>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(cap > 48 * 1024 ? cap : 48 * 1024));
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

cudaError_t prepare_mf_start() {
    // one limit for every batch: the largest instance's
    return cudaFuncSetAttribute(mf_start_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mf_smem_bytes(kBatchMaxN));
}

cudaError_t launch_mf_start(const float2* coords, uint32_t* routes, const BatchInstance* inst,
                            const uint32_t* order, uint32_t count, uint32_t max_n, int sms,
                            cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    const uint32_t grid = std::min<uint32_t>(count, (uint32_t)(sms > 0 ? sms : 1) * 4u);
    mf_start_kernel<<<grid, kMfThreads, mf_smem_bytes(max_n), s>>>(coords, routes, inst, order,
                                                                  count, max_n);
    return cudaGetLastError();
}

cudaError_t launch_start_tour(const float2* xy, uint32_t n, int kind, uint32_t* route,
                              cudaStream_t s) {
    if (n == 0 || n > kBatchMaxN || (kind != kStartNN && kind != kStartMF))
        return cudaErrorInvalidValue;
    const size_t cap = std::max<size_t>(mf_smem_bytes(kBatchMaxN), sizeof(uint32_t) * kBatchMaxN);
    cudaError_t e = cudaFuncSetAttribute(start_tour_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    if (e != cudaSuccess) return e;
    const size_t smem = kind == kStartNN ? sizeof(uint32_t) * n : mf_smem_bytes(n);
    start_tour_kernel<<<1, kMfThreads, smem, s>>>(xy, n, kind, route);
    return cudaGetLastError();
}

}  // namespace logo
