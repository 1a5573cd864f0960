// Cooperative persistent descent for small tours (n <= kCoopMaxN = 6,144),
// sm_103a.
//
// The multi-kernel descent launches a sweep and a gather per move; for small
// and mid-size tours those two launches (10 us and 5 us at n = 1000) are
// mostly latency, not work.  Here one cooperative launch runs the whole
// descent: every CTA holds the ordered tour (x, y, incoming edge, city id in
// the spare field) in its own shared memory, the CTAs' warps share the
// sweep's warp tiles (sweep_core.cuh, MUFU screen, exact re-evaluation), the
// per-CTA best keys meet in one 64-bit atomicMin per move, and after one grid
// barrier every CTA reads the same best move and applies it to its own copy
// (rotate + reverse in place: rev[p,q) || rev[q,n), then rev[0,q), as in
// cta_tour.cuh).  Per move: one barrier, no global tour traffic.
//
// Move semantics, candidate set, tie rule and the DevState bookkeeping are
// those of sweep.cu + apply_move_kernel (src/solvers/twoOptLocalSolver.cpp:
// 22-64): moves, total_moves, sweeps (+1 for the converging sweep), the move
// log, kErrMoveLimit at max_moves, kErrBadKey on an out-of-range key.  The
// final tour is written back to buffer `cur` by CTA 0.
//
// Best-key slots rotate over three entries: sweep s of the launch uses slot
// s % 3, and before arriving at barrier s CTA 0 clears slot (s + 1) % 3,
// which every CTA finished reading before it arrived at barrier s - 1.
// Counting sweeps rather than moves lets one launch run several descents
// back to back (the ILS launch: descent, length, accept/revert, kick, ...).  Barrier waits are
// bounded (2 s of %globaltimer); a CTA that gives up sets kErrTimeout and
// leaves the loop, so the others give up too and the launch ends.
#include "logo_device.cuh"
#include "logo_internal.h"
#include "neighbour_core.cuh"
#include "sweep_core.cuh"

namespace logo {

namespace {

constexpr unsigned long long kCoopWaitNs = 2000000000ull;
constexpr uint32_t kCoopSmallN = 2500;  // 256-thread CTAs up to here, 512 above

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned int* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier (generation counter); false when the wait ran out.
__device__ bool grid_barrier(CoopSync* cs, unsigned int nblocks, DevState* st, bool* ok_s) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int g = ld_acquire_u32(&cs->gen);
        __threadfence();
        const unsigned int t = atomicAdd(&cs->count, 1u);
        bool ok = true;
        if (t == nblocks - 1) {
            atomicExch(&cs->count, 0u);
            __threadfence();
            atomicAdd(&cs->gen, 1u);
        } else {
            const unsigned long long t0 = global_timer_ns();
            while (ld_acquire_u32(&cs->gen) == g) {
                if (global_timer_ns() - t0 > kCoopWaitNs) {
                    atomicOr(&st->status, kErrTimeout);
                    ok = false;
                    break;
                }
                __nanosleep(32);
            }
        }
        // as cooperative groups' grid sync: after the barrier every thread
        // sees every global write made before it (the cooperative neighbour
        // phase reads the tour other SMs just moved)
        __threadfence();
        *ok_s = ok;
    }
    __syncthreads();
    return *ok_s;
}

// Reverses [a0, a1) and [b0, b1) (disjoint) of the shared tour in one pass.
template <int NT>
__device__ __forceinline__ void reverse2_f4(float4* T, uint32_t a0, uint32_t a1, uint32_t b0,
                                            uint32_t b1) {
    const uint32_t ha = (a1 - a0) / 2, hb = (b1 - b0) / 2;
    for (uint32_t t = threadIdx.x; t < ha + hb; t += NT) {
        uint32_t x, y;
        if (t < ha) {
            x = a0 + t;
            y = a1 - 1 - t;
        } else {
            x = b0 + (t - ha);
            y = b1 - 1 - (t - ha);
        }
        const float4 vx = T[x], vy = T[y];
        T[x] = vy;
        T[y] = vx;
    }
}

// Sum over the CTA (every thread returns the total).
template <int NT>
__device__ __forceinline__ unsigned long long cta_sum(unsigned long long v,
                                                      unsigned long long* part) {
    v = warp_sum_u64(v);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long t = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) t += part[w];
    __syncthreads();
    return t;
}

// Exact incoming edge of every position of the shared tour.
template <int NT>
__device__ __forceinline__ void recompute_edges(OrderedCity* Q, uint32_t n) {
    for (uint32_t k = threadIdx.x; k < n; k += NT) {
        const OrderedCity a = Q[k];
        const OrderedCity b = Q[k == 0 ? n - 1 : k - 1];
        Q[k].e = (float)exact_dist(b.x, b.y, a.x, a.y);
    }
    __syncthreads();
}

// ILS == false: one descent (the multi-kernel descent's bookkeeping).
// ILS == true: a whole ILS call.  Every CTA keeps the best tour's city ids in
// shared memory and runs the same length, accept/revert and kick on its own
// copy (ILSGlobalSolverSequential.cpp:87-94, ILSGlobalSolver.cpp:37-48 and
// the double bridge), so those steps need no grid barrier; the sweeps of
// consecutive descents take the best-key slots by a running sweep count.
template <int R, int TC, int NT, bool ILS>
__global__ void __launch_bounds__(NT) coop_descent_kernel(CoopArgs A) {
    constexpr int kCoopThreads = NT;
    constexpr int kCoopWarps = NT / 32;
    extern __shared__ __align__(16) unsigned char coop_smem[];
    OrderedCity* Q = reinterpret_cast<OrderedCity*>(coop_smem);
    const uint32_t n = A.n;
    constexpr uint32_t RT = 32 * R;
    const uint32_t nrb = (n - 3 + RT - 1) / RT;  // row blocks over rows 1..n-3
    uint32_t* tbl = reinterpret_cast<uint32_t*>(coop_smem + (size_t)n * sizeof(OrderedCity));
    uint32_t* sbest = tbl + (nrb + 2);  // ILS: city ids of the best tour
    __shared__ unsigned long long wbest[kCoopWarps];
    __shared__ unsigned long long psum[kCoopWarps];
    __shared__ bool bar_ok;
    DevState* st = A.st;
    CoopSync* cs = A.cs;
    // set before the launch and identical for every CTA
    if (*(volatile unsigned int*)&st->converged) return;
    const uint32_t cur = *(volatile unsigned int*)&st->cur;
    OrderedCity* Qg = cur ? A.Q1 : A.Q0;
    uint32_t* Rg = cur ? A.R1 : A.R0;
    for (uint32_t k = threadIdx.x; k < n; k += kCoopThreads) {
        OrderedCity o = Qg[k];
        o.pad = __uint_as_float(Rg[k]);
        Q[k] = o;
        if (ILS) sbest[k] = A.route_best[k];
    }
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        tbl[0] = 0;
        for (uint32_t b = 0; b < nrb; ++b) {
            const uint32_t row0 = 1 + b * RT;
            acc += (n - row0 - 2 + TC - 1) / TC;
            tbl[b + 1] = acc;
        }
    }
    __syncthreads();
    const uint32_t total = tbl[nrb];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long m0 = *(volatile unsigned long long*)&st->moves;
    const unsigned long long maxm = *(volatile unsigned long long*)&st->max_moves;
    unsigned long long m = 0, sweeps = 0, seq = 0, total_m = 0;
    unsigned long long best_len = 0, accepted = 0, kicks = 0;
    uint64_t rng = 0;
    if (ILS) {
        best_len = *(volatile unsigned long long*)&st->best_length;
        rng = *(volatile unsigned long long*)&st->rng;
    }
    bool limit = false, bad = false, failed = false;
    float4* T = reinterpret_cast<float4*>(Q);
    for (uint32_t it = 0;; ++it) {
        m = 0;
        for (;;) {
            // sweep: warp tiles dealt over every warp of the grid
            uint64_t best = kNoMove;
            for (uint32_t t = blockIdx.x * kCoopWarps + warp; t < total;
                 t += gridDim.x * kCoopWarps) {
                uint32_t lo = 0, hi = nrb;  // row block b with tbl[b] <= t < tbl[b + 1]
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) / 2;
                    if (tbl[mid] <= t) lo = mid; else hi = mid;
                }
                const uint32_t row0 = 1 + lo * RT;
                const uint32_t col0 = row0 + 2 + (t - tbl[lo]) * TC;
                const uint32_t col1 = min(col0 + TC, n);
                const uint32_t ib = row0 + lane * R;
                int B = -1;
                if (best != kNoMove) B = min(B, key_delta(best));
                RowBlock<R> rb;
                load_rows<R>(rb, Q, ib, n);
                refresh_thresholds<R>(rb, Q, ib, n, B, A.margin);
                walk_columns<R>(rb, Q, 0, col0, col1, ib, n, Q, A.margin, B, best);
            }
            best = warp_min_u64(best);
            if (lane == 0) wbest[warp] = best;
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned long long k = wbest[0];
#pragma unroll
                for (int w = 1; w < kCoopWarps; ++w) k = wbest[w] < k ? wbest[w] : k;
                if (k != kNoMove) atomicMin(&cs->slot[seq % 3], k);
                if (blockIdx.x == 0) cs->slot[(seq + 1) % 3] = kNoMove;
            }
            if (!grid_barrier(cs, gridDim.x, st, &bar_ok)) {
                failed = true;
                break;
            }
            ++sweeps;
            const unsigned long long key = ld_acquire_u64(&cs->slot[seq % 3]);
            ++seq;
            if (key == kNoMove) break;  // local optimum
            // reported move (i, j+1): p = i < q = j+1 (twoOptLocalSolver.cpp:41-48)
            const uint32_t p = key_i(key), q = key_j(key);
            if (!(p >= 1 && q < n && q >= p + 2)) {
                bad = true;
                break;
            }
            if (!ILS && blockIdx.x == 0 && threadIdx.x == 0) {
                int* log = st->move_log;
                const unsigned long long idx = m0 + m;
                if (log && idx < st->log_cap) {
                    log[3 * idx + 0] = key_delta(key);
                    log[3 * idx + 1] = (int)p;
                    log[3 * idx + 2] = (int)q;
                }
            }
            // new = old[p..q) ++ rev(old[0..p)) ++ rev(old[q..n))
            reverse2_f4<NT>(T, p, q, q, n);
            __syncthreads();
            reverse2_f4<NT>(T, 0, q, 0, 0);
            __syncthreads();
            recompute_edges<NT>(Q, n);
            ++m;
            if (m0 + m >= maxm) {
                limit = true;
                break;
            }
        }
        total_m += m;
        if (!ILS || failed || bad) break;
        // length of this CTA's copy; keep it if strictly shorter, else revert
        unsigned long long part = 0;
        for (uint32_t k = threadIdx.x; k < n; k += kCoopThreads)
            part += (unsigned long long)Q[k].e;
        const unsigned long long len = cta_sum<NT>(part, psum);
        if (len < best_len) {
            for (uint32_t k = threadIdx.x; k < n; k += kCoopThreads)
                sbest[k] = __float_as_uint(Q[k].pad);
            best_len = len;
            ++accepted;
        } else {
            for (uint32_t k = threadIdx.x; k < n; k += kCoopThreads) {
                const uint32_t id = sbest[k];
                const float2 c = A.xy[id];
                Q[k] = OrderedCity{c.x, c.y, 0.f, __uint_as_float(id)};
            }
            __syncthreads();
            recompute_edges<NT>(Q, n);
        }
        __syncthreads();
        if (it == A.kicks) break;
        // kick (the same draws as kick_kernel in tour.cu)
        if (A.kick_kind == 1) {
            uint32_t c[3];
            for (int k = 0; k < 3; ++k) c[k] = 1 + uniform_below(rng, n - 1);
            uint32_t t;
            if (c[1] < c[0]) { t = c[0]; c[0] = c[1]; c[1] = t; }
            if (c[2] < c[1]) { t = c[1]; c[1] = c[2]; c[2] = t; }
            if (c[1] < c[0]) { t = c[0]; c[0] = c[1]; c[1] = t; }
            // old[0,p1) old[p2,p3) old[p1,p2) old[p3,n): swap two adjacent blocks
            reverse2_f4<NT>(T, c[0], c[1], c[1], c[2]);
            __syncthreads();
            reverse2_f4<NT>(T, c[0], c[2], 0, 0);
        } else {
            uint32_t a = uniform_below(rng, n);
            uint32_t b = uniform_below(rng, n);
            if (b < a) { const uint32_t t = a; a = b; b = t; }
            // rotate by a, reverse [b - a, n): old[a,b) ++ rev(old[0,a)) ++ rev(old[b,n))
            reverse2_f4<NT>(T, a, b, b, n);
            __syncthreads();
            reverse2_f4<NT>(T, 0, b, 0, 0);
        }
        __syncthreads();
        recompute_edges<NT>(Q, n);
        ++kicks;
        m0 = 0;
    }
    if (blockIdx.x == 0 && !failed) {
        for (uint32_t k = threadIdx.x; k < n; k += kCoopThreads) {
            OrderedCity o = Q[k];
            const uint32_t id = __float_as_uint(o.pad);
            o.pad = 0.f;
            Rg[k] = id;
            Qg[k] = o;
            if (ILS) {
                A.route_best[k] = id;
                A.Qbest[k] = o;
            }
        }
        if (threadIdx.x == 0) {
            st->moves = m0 + m;
            st->total_moves += total_m;
            st->sweeps += sweeps;
            st->best_key = kNoMove;
            st->converged = 1;
            if (ILS) {
                st->rng = rng;
                st->best_length = best_len;
                st->accepted += accepted;
                st->kicks += kicks;
            }
            if (limit) atomicOr(&st->status, kErrMoveLimit);
            if (bad) atomicOr(&st->status, kErrBadKey);
        }
    }
}

template <int R, int TC, bool ILS>
size_t coop_smem(uint32_t n) {
    const uint32_t nrb = (n - 3 + 32 * R - 1) / (32 * R);
    return (size_t)n * sizeof(OrderedCity) + sizeof(uint32_t) * (nrb + 2) +
           (ILS ? sizeof(uint32_t) * (size_t)n : 0);
}

// Grid for a cooperative launch: every CTA resident at once (occupancy x
// SMs), and no more CTAs than the sweep has warp tiles for.
template <int R, int TC, int NT, bool ILS>
int coop_grid_t(uint32_t n, uint32_t max_n, int device) {
    const size_t smem = coop_smem<R, TC, ILS>(n);
    // the limit is shared by every context: set it for the largest n this
    // instantiation runs, not for this context's n
    if (cudaFuncSetAttribute(coop_descent_kernel<R, TC, NT, ILS>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)coop_smem<R, TC, ILS>(max_n)) != cudaSuccess)
        return 0;
    int per_sm = 0, sms = 0, coop = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coop_descent_kernel<R, TC, NT, ILS>,
                                                      NT, smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess)
        return 0;
    if (!coop || per_sm < 1) return 0;
    constexpr uint32_t RT = 32 * R;
    uint64_t tiles = 0;
    for (uint32_t row0 = 1; row0 + 3 <= n; row0 += RT) tiles += (n - row0 - 2 + TC - 1) / TC;
    const uint64_t want = (tiles + NT / 32 - 1) / (NT / 32);
    const uint64_t cap = (uint64_t)per_sm * sms;
    return (int)(want < cap ? (want < 1 ? 1 : want) : cap);
}

template <int R, int TC, int NT, bool ILS>
cudaError_t launch_coop_t(const CoopArgs& A, int grid, cudaStream_t s) {
    CoopArgs a = A;
    void* args[] = {&a};
    return cudaLaunchCooperativeKernel((const void*)coop_descent_kernel<R, TC, NT, ILS>,
                                       dim3(grid), dim3(NT), args,
                                       coop_smem<R, TC, ILS>(A.n), s);
}

// Test hook for the bounded wait: one CTA waits at a barrier sized for two,
// which nothing else will reach; the wait gives up after its budget and sets
// kErrTimeout in st->status.
// The neighbour phase of LOGO_SEARCH_NEIGHBOUR(_OROPT) as one cooperative
// launch over tours of any size (the tour stays in global memory, buffers
// cur and cur ^ 1 as for the multi-kernel path): per move, every CTA
// evaluates the candidates of its positions (neighbour_core.cuh) into the
// move's key slots, one grid barrier, every CTA reads the same best move
// (the rule of apply_nbr_move_kernel) and gathers its share of the moved
// tour (Q, route, pos), a second barrier, and the buffers swap.  Slot s % 3
// of sweep s is cleared by CTA 0 during sweep s - 1, after every CTA read it
// for sweep s - 3.  DevState at the end is what the sweep and apply kernels
// leave after the same moves: moves, total_moves, sweeps and nbr_sweeps
// (one per sweep, the converging one included), converged, cur, the move
// log, kErrMoveLimit at max_moves, kErrBadKey on an out-of-range key.
#ifndef LOGO_COOP_LD
#define LOGO_COOP_LD kLdCoherent
#endif
constexpr int kCoopLd = LOGO_COOP_LD;

template <bool OR, int NT>
__global__ void __launch_bounds__(NT) coop_nbr_kernel(NbrLaunch L, CoopSync* cs) {
    __shared__ unsigned long long red[NT / 32];
    __shared__ unsigned long long red_or[OR ? kOrSlots : 1][NT / 32];
    __shared__ bool ok_s;
    DevState* st = L.st;
    const uint32_t n = L.n;
    const unsigned int nblocks = gridDim.x;
    uint32_t cur = *(volatile unsigned int*)&st->cur;
    const unsigned long long max_moves = *(volatile unsigned long long*)&st->max_moves;
    unsigned long long moves = *(volatile unsigned long long*)&st->moves;
    const unsigned long long moves0 = moves;
    const bool start_done = *(volatile unsigned int*)&st->converged;
    uint32_t sweeps = 0;
    bool limit = false, bad = false, timeout = false;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t sw = 0; !start_done; ++sw) {
        const uint32_t slot = sw % 3;
        const OrderedCity* Q = cur ? L.Q1 : L.Q0;
        const uint32_t* R = cur ? L.R1 : L.R0;
        uint64_t best = kNoMove;
        uint64_t bo[kOrSlots];
#pragma unroll
        for (int v = 0; v < kOrSlots; ++v) bo[v] = kNoMove;
        for (uint32_t i = blockIdx.x * NT + threadIdx.x; i < n; i += nblocks * NT)
            nbr_position<OR, kCoopLd>(i, Q, R, L.pos, L.nbr, L.K, n, L.margin, best, bo);
        best = warp_min_u64(best);
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
            if (m != kNoMove) atomicMin(&cs->slot[slot], (unsigned long long)m);
            if (OR) {
                for (int v = 0; v < kOrSlots; ++v) {
                    uint64_t mv = red_or[v][0];
                    for (int w = 1; w < NT / 32; ++w) mv = red_or[v][w] < mv ? red_or[v][w] : mv;
                    if (mv != kNoMove) atomicMin(&cs->or_slot[slot][v], (unsigned long long)mv);
                }
            }
            if (blockIdx.x == 0) {  // the next sweep's slots
                const uint32_t nx = (sw + 1) % 3;
                cs->slot[nx] = kNoMove;
                for (int v = 0; v < kOrSlots; ++v) cs->or_slot[nx][v] = kNoMove;
            }
        }
        ++sweeps;
        if (!grid_barrier(cs, nblocks, st, &ok_s)) {
            timeout = true;
            break;
        }
        // the move: lowest delta, ties to the 2-opt move, then the lower slot
        uint64_t key = ld_acquire_u64(&cs->slot[slot]);
        int vslot = -1;
        if (OR) {
            for (int v = 0; v < kOrSlots; ++v) {
                const uint64_t k = ld_acquire_u64(&cs->or_slot[slot][v]);
                if (k != kNoMove && (key == kNoMove || key_delta(k) < key_delta(key))) {
                    key = k;
                    vslot = v;
                }
            }
        }
        if (key == kNoMove) break;  // converged (every CTA reads the same keys)
        const uint32_t a = key_i(key), b = key_j(key);
        const uint32_t Lg = vslot >= 0 ? or_len(vslot) : 0u;
        const bool rev = vslot >= 0 && or_rev(vslot);
        const bool ok = vslot < 0 ? (a >= 1 && b < n && b >= a + 2)
                                  : (a >= 1 && a + Lg <= n - 1 &&
                                     (b + 2 <= a || (b >= a + Lg && b + 2 <= n)));
        if (!ok) {
            bad = true;
            break;
        }
        const OrderedCity* Qs = Q;
        OrderedCity* Qd = cur ? L.Q0w : L.Q1w;
        uint32_t* Rd = cur ? L.R0w : L.R1w;
        for (uint32_t k = blockIdx.x * NT + threadIdx.x; k < n; k += nblocks * NT) {
            const uint32_t km = k == 0 ? n - 1 : k - 1;
            const uint32_t src = vslot < 0 ? rotrev_src(k, a, b, n) : oropt_src(k, a, Lg, b, rev);
            const uint32_t srcm =
                vslot < 0 ? rotrev_src(km, a, b, n) : oropt_src(km, a, Lg, b, rev);
            const OrderedCity qa = ld_city<kCoopLd>(Qs + src), qb = ld_city<kCoopLd>(Qs + srcm);
            OrderedCity o;
            o.x = qa.x;
            o.y = qa.y;
            o.e = (float)exact_dist(qb.x, qb.y, qa.x, qa.y);
            o.pad = 0.f;
            Qd[k] = o;
            const uint32_t id = ld_u32<kCoopLd>(R + src);
            Rd[k] = id;
            L.pos[min(id, n - 1)] = k;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0 && st->move_log && moves < st->log_cap) {
            st->move_log[3 * moves + 0] = key_delta(key);
            st->move_log[3 * moves + 1] = vslot < 0 ? (int)a : -1 - (int)(a + ((uint32_t)vslot << 21));
            st->move_log[3 * moves + 2] = (int)b;
        }
        ++moves;
        cur ^= 1u;
        if (moves >= max_moves) limit = true;
        if (!grid_barrier(cs, nblocks, st, &ok_s)) {
            timeout = true;
            break;
        }
        if (limit) break;
    }
    // leave the key slots empty for the next launch (a graph replays this
    // one without a memset in between): every CTA has read its last slot
    // once all have passed one more barrier
    if (!timeout && grid_barrier(cs, nblocks, st, &ok_s) && blockIdx.x == 0 &&
        threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            cs->slot[k] = kNoMove;
            for (int v = 0; v < kOrSlots; ++v) cs->or_slot[k][v] = kNoMove;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long made = moves - moves0;
        st->moves = moves;
        st->total_moves += made;
        st->sweeps += made + (limit || timeout || bad || start_done ? 0 : 1);
        st->nbr_sweeps += sweeps;
        st->cur = cur;
        st->best_key = kNoMove;
        for (int v = 0; v < kOrSlots; ++v) st->or_key[v] = kNoMove;
        st->converged = 1;
        if (limit) atomicOr(&st->status, kErrMoveLimit);
        if (bad) atomicOr(&st->status, kErrBadKey);
    }
}

__global__ void barrier_probe_kernel(CoopSync* cs, DevState* st) {
    __shared__ bool ok;
    grid_barrier(cs, 2u, st, &ok);
}

}  // namespace

cudaError_t launch_barrier_probe(CoopSync* cs, DevState* st, cudaStream_t s) {
    barrier_probe_kernel<<<1, 32, 0, s>>>(cs, st);
    return cudaGetLastError();
}

// Warp tiles of 64 rows x 32 columns; 256-thread CTAs up to 2,500 cities,
// 512 above (measured on GB300, random tours, microseconds per move: n = 1000
// 10.4 with 256 threads vs 11.3 with 512, n = 3000 12.7 with 512; the
// graph-driven descent 16.7 and 29.2; 4-row x 64-column tiles leave most SMs
// idle at n = 3000, 24.6.  From about 8,000 cities on the graph-driven
// descent is as fast or faster, so the limit is 6,144).
int coop_grid(uint32_t n, int device) {
    if (n < 8 || n > kCoopMaxN) return 0;
    return n <= kCoopSmallN ? coop_grid_t<2, 32, 256, false>(n, kCoopSmallN, device)
                            : coop_grid_t<2, 32, 512, false>(n, kCoopMaxN, device);
}

int coop_ils_grid(uint32_t n, int device) {
    if (n < 8 || n > kCoopMaxN) return 0;
    return n <= kCoopSmallN ? coop_grid_t<2, 32, 256, true>(n, kCoopSmallN, device)
                            : coop_grid_t<2, 32, 512, true>(n, kCoopMaxN, device);
}

cudaError_t launch_coop_descent(const CoopArgs& A, int grid, cudaStream_t s) {
    return A.n <= kCoopSmallN ? launch_coop_t<2, 32, 256, false>(A, grid, s)
                              : launch_coop_t<2, 32, 512, false>(A, grid, s);
}

cudaError_t launch_coop_ils(const CoopArgs& A, int grid, cudaStream_t s) {
    return A.n <= kCoopSmallN ? launch_coop_t<2, 32, 256, true>(A, grid, s)
                              : launch_coop_t<2, 32, 512, true>(A, grid, s);
}

template <bool OR, int NT>
static int coop_nbr_grid_t(int device) {
    int per_sm = 0, sms = 0, coop = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coop_nbr_kernel<OR, NT>, NT, 0) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess)
        return 0;
    if (!coop || per_sm < 1) return 0;
    return per_sm * sms;
}

int coop_nbr_grid(uint32_t n, bool oropt, int device) {
    const int nt = oropt ? 128 : 256;
    const int cap = oropt ? coop_nbr_grid_t<true, 128>(device) : coop_nbr_grid_t<false, 256>(device);
    const int want = (int)((n + nt - 1) / nt);
    return cap < 1 ? 0 : (want < cap ? (want < 1 ? 1 : want) : cap);
}

cudaError_t launch_coop_nbr(const NbrLaunch& L, CoopSync* cs, int grid, cudaStream_t s) {
    // a cooperative launch through the launch attribute, which stream capture
    // records as a cooperative kernel node (the device-run ILS graph)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(L.oropt ? 128u : 256u);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (L.oropt) return cudaLaunchKernelEx(&cfg, coop_nbr_kernel<true, 128>, L, cs);
    return cudaLaunchKernelEx(&cfg, coop_nbr_kernel<false, 256>, L, cs);
}

}  // namespace logo
