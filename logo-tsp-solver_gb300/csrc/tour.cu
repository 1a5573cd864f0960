// Device-resident tour maintenance: tour-ordered gather, 2-opt move
// application, tour length, ILS kicks and accept/revert (sm_103a).
//
// The tour lives in two buffers (Q[cur], route[cur]); every permutation is a
// gather from buffer cur into buffer cur^1 followed by a flip of cur made by
// the last CTA to finish (threadfence + counter, no spinning), so the host
// never touches the tour between moves.  Where the context keeps city
// positions (the boxed sweep's seed pass, the neighbour search), every
// kernel that moves the tour writes them too; a position left stale (the
// cooperative exhaustive descent does not write them) only weakens the
// seed, never a result, because the seed pass evaluates whatever pair of
// positions it reads exactly, and the neighbour search recomputes them
// before its first use.
//   load_route_kernel      ≙ ordered-coordinate gather, CUDASolver.cpp:316-319
//   apply_move_kernel      ≙ rotate + reverse, twoOptLocalSolver.cpp:41-48
//   tour_length_kernel     ≙ routeLength, headers.h:170-189
//   kick_kernel            ≙ ILSGlobalSolver::kick, ILSGlobalSolver.cpp:37-48
//                            (and the double bridge, which has no reference)
//   accept_kernel          ≙ accept/revert, ILSGlobalSolverSequential.cpp:87-94
#include <cstdlib>

#include "logo_device.cuh"
#include "logo_internal.h"

namespace logo {

bool chained_launch_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("LOGO_CHAINED_LAUNCH");
        return !(e && e[0] == '0');
    }();
    return on;
}

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(uint32_t n) {
    unsigned g = (n + kThreads - 1) / kThreads;
    return g < 1 ? 1 : (g > 4096 ? 4096 : g);
}

// Last-CTA election: true in exactly one thread of the grid, after every
// CTA has finished its writes.  The CTA barrier orders its threads' writes
// before thread 0's fence, which then makes them visible device-wide before
// the counter moves (one fence per CTA, not one per thread: measured on
// GB300 the per-thread fences were a tenth of the gather's stalls).
__device__ __forceinline__ bool last_block_done(unsigned int* counter) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        *counter = 0;
        return true;
    }
    return false;
}

// Loads a tour from src (the caller's buffer read in place, or a device
// copy of it): route[0] = src (when src is not route[0] itself), Q[0] =
// the ordered cities with their incoming edges, pos = the position of every
// city, and the permutation check: seen[v] holds the number of the last
// load that met city v, so a city met twice in this load (or an id >= n)
// makes the route bad without clearing anything between loads.  The last
// CTA to finish sets st->bad_route and st->cur = 0 and, with
// reset_moves != 0, prepares a descent (the fields reset_descent_kernel
// sets; nothing to descend on a bad route).  Out-of-range ids are read as
// city 0 for the coordinates.
__global__ void load_route_kernel(const float2* __restrict__ xy, const uint32_t* src,
                                  uint32_t* R0, OrderedCity* __restrict__ Q, uint32_t n,
                                  uint32_t* __restrict__ seen, uint32_t epoch,
                                  uint32_t* __restrict__ pos, DevState* st,
                                  unsigned long long reset_moves) {
    chain_wait();
    chain_release();
    bool bad = false;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += gridDim.x * blockDim.x) {
        const uint32_t raw = src[k], rawp = src[k == 0 ? n - 1 : k - 1];
        bool b = raw >= n;
        if (!b) b = atomicExch(&seen[raw], epoch) == epoch;
        bad |= b;
        if (!b && pos) pos[raw] = k;
        if (R0 != src) R0[k] = raw;
        const uint32_t v = raw < n ? raw : 0u, w = rawp < n ? rawp : 0u;
        const float2 a = xy[v];
        const float2 c = xy[w];
        OrderedCity o;
        o.x = a.x;
        o.y = a.y;
        o.e = (float)exact_dist(c.x, c.y, a.x, a.y);
        o.pad = 0.f;
        Q[k] = o;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&st->load_bad, 1u);
    if (last_block_done(&st->done_blocks)) {
        const unsigned int b = atomicExch(&st->load_bad, 0u);
        st->bad_route = b;
        st->cur = 0u;
        if (reset_moves) {
            st->best_key = kNoMove;
            for (int v = 0; v < kOrSlots; ++v) st->or_key[v] = kNoMove;
            st->moves = 0;
            st->nbr_sweeps = 0;
            st->status = 0u;
            st->converged = b ? 1u : 0u;
            st->sweeps_at_reset = st->sweeps;
            st->max_moves = reset_moves;
        }
    }
}

// Writes the current tour (or the best one) to dst, the caller's buffer
// written in place.
__global__ void store_route_kernel(const uint32_t* __restrict__ R0,
                                   const uint32_t* __restrict__ R1,
                                   const uint32_t* __restrict__ Rbest, uint32_t* dst,
                                   uint32_t n, const DevState* st, int best) {
    chain_wait();
    chain_release();
    const uint32_t* R = best ? Rbest : (*(volatile const unsigned int*)&st->cur ? R1 : R0);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += gridDim.x * blockDim.x)
        dst[k] = R[k];
}

__global__ void reset_descent_kernel(DevState* st, unsigned long long max_moves) {
    chain_wait();
    chain_release();
    st->best_key = kNoMove;
    for (int v = 0; v < kOrSlots; ++v) st->or_key[v] = kNoMove;
    st->moves = 0;
    st->nbr_sweeps = 0;
    st->status = 0u;
    st->converged = st->bad_route ? 1u : 0u;  // nothing to descend on a bad route
    st->sweeps_at_reset = st->sweeps;
    st->done_blocks = 0;
    st->max_moves = max_moves;
}

// Gather new[k] = old[src(k)] for a permutation given by its source map,
// recomputing the incoming edge lengths.
template <typename Src>
__device__ __forceinline__ void gather_tour(const OrderedCity* __restrict__ Qs,
                                            const uint32_t* __restrict__ Rs,
                                            OrderedCity* __restrict__ Qd,
                                            uint32_t* __restrict__ Rd, uint32_t n,
                                            uint32_t* __restrict__ pos, Src src,
                                            uint32_t* out = nullptr) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += gridDim.x * blockDim.x) {
        const uint32_t s = src(k);
        const uint32_t sp = src(k == 0 ? n - 1 : k - 1);
        const OrderedCity a = Qs[s];
        const OrderedCity b = Qs[sp];
        OrderedCity o;
        o.x = a.x;
        o.y = a.y;
        o.e = (float)exact_dist(b.x, b.y, a.x, a.y);
        o.pad = 0.f;
        Qd[k] = o;
        const uint32_t id = Rs[s];
        Rd[k] = id;
        if (out) out[k] = id;
        if (pos) pos[min(id, n - 1)] = k;
    }
}

// out (optional): the caller's route buffer, written with the tour this
// launch leaves (moved, or unchanged when there is no move) -- the last step
// of a short descent hands its result back without a separate store.
__global__ void apply_move_kernel(TourBufs T, uint32_t* out) {
    chain_wait();
    chain_release();
    DevState* st = T.st;
    const uint32_t cur = *(volatile unsigned int*)&st->cur;
    const uint32_t n = T.n;
    const bool done = *(volatile unsigned int*)&st->converged;
    const uint64_t key = done ? kNoMove : *(volatile unsigned long long*)&st->best_key;
    if (key == kNoMove) {
        if (out) {
            const uint32_t* R = cur ? T.route[1] : T.route[0];
            for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
                 k += gridDim.x * blockDim.x)
                out[k] = R[k];
        }
        if (!done && blockIdx.x == 0 && threadIdx.x == 0) {
            st->converged = 1;
            st->sweeps += 1;
        }
        return;
    }
    // reported move (i, j+1): p = i < q = j+1 (twoOptLocalSolver.cpp:41-48)
    const uint32_t p = key_i(key), q = key_j(key);
    if (!(p >= 1 && q < n && q >= p + 2)) {
        if (out) {
            const uint32_t* R = cur ? T.route[1] : T.route[0];
            for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n;
                 k += gridDim.x * blockDim.x)
                out[k] = R[k];
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            atomicOr(&st->status, kErrBadKey);
            st->converged = 1;
        }
        return;
    }
    gather_tour(cur ? T.Q[1] : T.Q[0], cur ? T.route[1] : T.route[0], cur ? T.Q[0] : T.Q[1],
                cur ? T.route[0] : T.route[1], n, T.pos,
                [=] __device__(uint32_t k) { return rotrev_src(k, p, q, n); }, out);
    if (last_block_done(&st->done_blocks)) {
        const unsigned long long m = st->moves;
        if (st->move_log && m < st->log_cap) {
            st->move_log[3 * m + 0] = key_delta(key);
            st->move_log[3 * m + 1] = (int)p;
            st->move_log[3 * m + 2] = (int)q;
        }
        st->moves = m + 1;
        st->total_moves += 1;
        st->sweeps += 1;
        st->best_key = kNoMove;
        st->cur = cur ^ 1;
        if (m + 1 >= st->max_moves) {
            st->converged = 1;
            atomicOr(&st->status, kErrMoveLimit);
        }
    }
}

__global__ void tour_length_kernel(TourBufs T) {
    DevState* st = T.st;
    const uint32_t cur = *(volatile unsigned int*)&st->cur;
    const OrderedCity* Q = cur ? T.Q[1] : T.Q[0];
    unsigned long long s = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T.n;
         k += gridDim.x * blockDim.x)
        s += (unsigned long long)Q[k].e;
    s = warp_sum_u64(s);
    __shared__ unsigned long long part[kThreads / 32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += part[w];
        atomicAdd(&st->length_acc, t);
    }
    if (last_block_done(&st->len_done)) {
        st->length = st->length_acc;
        st->length_acc = 0;
    }
}

// kind < 0: the kind stored in st->kick_kind (the device-run ILS graph).
__global__ void kick_kernel(TourBufs T, int kind) {
    DevState* st = T.st;
    if (kind < 0) kind = (int)*(volatile unsigned int*)&st->kick_kind;
    const uint32_t cur = *(volatile unsigned int*)&st->cur;
    uint64_t rng = *(volatile unsigned long long*)&st->rng;
    const uint32_t n = T.n;
    if (kind == 1) {
        uint32_t c[3];
        for (int k = 0; k < 3; ++k) c[k] = 1 + uniform_below(rng, n - 1);
        uint32_t t;
        if (c[1] < c[0]) { t = c[0]; c[0] = c[1]; c[1] = t; }
        if (c[2] < c[1]) { t = c[1]; c[1] = c[2]; c[2] = t; }
        if (c[1] < c[0]) { t = c[0]; c[0] = c[1]; c[1] = t; }
        const uint32_t p1 = c[0], p2 = c[1], p3 = c[2];
        gather_tour(cur ? T.Q[1] : T.Q[0], cur ? T.route[1] : T.route[0], cur ? T.Q[0] : T.Q[1],
                    cur ? T.route[0] : T.route[1], n, T.pos,
                    [=] __device__(uint32_t k) { return bridge_src(k, p1, p2, p3); });
    } else {
        uint32_t a = uniform_below(rng, n);
        uint32_t b = uniform_below(rng, n);
        if (b < a) { uint32_t t = a; a = b; b = t; }
        gather_tour(cur ? T.Q[1] : T.Q[0], cur ? T.route[1] : T.route[0], cur ? T.Q[0] : T.Q[1],
                    cur ? T.route[0] : T.route[1], n, T.pos,
                    [=] __device__(uint32_t k) { return rotrev_src(k, a, b, n); });
    }
    if (last_block_done(&st->done_blocks)) {
        st->rng = rng;
        st->cur = cur ^ 1;
        st->kicks += 1;
        st->best_key = kNoMove;
        for (int v = 0; v < kOrSlots; ++v) st->or_key[v] = kNoMove;
        st->moves = 0;
        st->converged = 0;
    }
}

// After a descent and tour_length_kernel: keep the tour if it is strictly
// shorter than the best so far, else restore the best.
__global__ void accept_kernel(TourBufs T) {
    DevState* st = T.st;
    const uint32_t cur = *(volatile unsigned int*)&st->cur;
    const unsigned long long len = *(volatile unsigned long long*)&st->length;
    const unsigned long long bl = *(volatile unsigned long long*)&st->best_length;
    const bool take = len < bl;
    OrderedCity* Qc = cur ? T.Q[1] : T.Q[0];
    uint32_t* Rc = cur ? T.route[1] : T.route[0];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T.n;
         k += gridDim.x * blockDim.x) {
        if (take) {
            T.Qbest[k] = Qc[k];
            T.route_best[k] = Rc[k];
        } else {
            Qc[k] = T.Qbest[k];
            const uint32_t id = T.route_best[k];
            Rc[k] = id;
            if (T.pos) T.pos[min(id, T.n - 1)] = k;
        }
    }
    if (last_block_done(&st->done_blocks)) {
        if (take) {
            st->best_length = len;
            st->accepted += 1;
        }
    }
}

__global__ void save_best_kernel(TourBufs T) {
    DevState* st = T.st;
    const uint32_t cur = *(volatile unsigned int*)&st->cur;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T.n;
         k += gridDim.x * blockDim.x) {
        T.Qbest[k] = (cur ? T.Q[1] : T.Q[0])[k];
        T.route_best[k] = (cur ? T.route[1] : T.route[0])[k];
    }
    if (last_block_done(&st->done_blocks)) {
        st->best_length = st->length;
        st->start_length = st->length;
    }
}

// Loop conditions of the device-run ILS graph (one thread each).  The
// descent loop runs while the tour has not converged and no error bit other
// than the move limit is set; every pass of its body applies at least one
// move or converges, so a pass that did neither stops the loop with
// kErrInternal.  Neither loop runs on a route that failed the permutation
// check.  The kick loop runs while fewer than kick_target kicks have
// been applied; each pass applies exactly one, so more passes than
// kick_target stop it with kErrInternal.  `first` marks the check in front
// of a loop (it resets the guard).
__global__ void descent_cond_kernel(DevState* st, cudaGraphConditionalHandle h, int first) {
    const unsigned int bad = (st->status & ~kErrMoveLimit) | st->bad_route;
    bool go = !st->converged && !bad;
    if (!first && go && st->moves == st->loop_mark) {
        atomicOr(&st->status, kErrInternal);
        go = false;
    }
    st->loop_mark = st->moves;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

__global__ void kick_cond_kernel(DevState* st, cudaGraphConditionalHandle h, int first) {
    const unsigned int bad = (st->status & ~kErrMoveLimit) | st->bad_route;
    bool go = st->kicks < st->kick_target && !bad;
    if (first) {
        st->ils_iters = 0;
    } else if (++st->ils_iters > st->kick_target) {
        atomicOr(&st->status, kErrInternal);
        go = false;
    }
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

}  // namespace

cudaError_t launch_descent_cond(DevState* st, cudaGraphConditionalHandle h, bool first,
                                cudaStream_t s) {
    descent_cond_kernel<<<1, 1, 0, s>>>(st, h, first ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_kick_cond(DevState* st, cudaGraphConditionalHandle h, bool first,
                             cudaStream_t s) {
    kick_cond_kernel<<<1, 1, 0, s>>>(st, h, first ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_load_route(const TourBufs& T, const uint32_t* src, uint32_t epoch,
                              unsigned long long reset_moves, cudaStream_t s) {
    return launch_chained(load_route_kernel, grid_for(T.n), kThreads, 0, s, T.xy, src,
                          T.route[0], T.Q[0], T.n, T.seen, epoch, T.pos, T.st, reset_moves);
}

cudaError_t launch_store_route(const TourBufs& T, uint32_t* dst, bool best, cudaStream_t s) {
    return launch_chained(store_route_kernel, grid_for(T.n), kThreads, 0, s, T.route[0],
                          T.route[1], T.route_best, dst, T.n, T.st, best ? 1 : 0);
}

cudaError_t launch_reset_descent(const TourBufs& T, unsigned long long max_moves,
                                 cudaStream_t s) {
    return launch_chained(reset_descent_kernel, 1, 1, 0, s, T.st, max_moves);
}
// The neighbour search with Or-opt moves: the lowest delta of the 2-opt
// candidate (st->best_key) and the five Or-opt slots, ties to the 2-opt
// move and then to the lower slot; applied as one gather (or marks
// convergence).  Trace entries of Or-opt moves are (delta, -1 - (s + slot *
// 2^21), p).
__global__ void apply_nbr_move_kernel(TourBufs T) {
    chain_wait();
    chain_release();
    DevState* st = T.st;
    if (*(volatile unsigned int*)&st->converged) return;
    const uint64_t key2 = *(volatile unsigned long long*)&st->best_key;
    int slot = -1;
    uint64_t key = key2;
    for (int v = 0; v < kOrSlots; ++v) {
        const uint64_t k = *(volatile unsigned long long*)&st->or_key[v];
        if (k != kNoMove && (key == kNoMove || key_delta(k) < key_delta(key))) {
            key = k;
            slot = v;
        }
    }
    const uint32_t cur = *(volatile unsigned int*)&st->cur;
    const uint32_t n = T.n;
    if (key == kNoMove) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->converged = 1;
            st->sweeps += 1;
        }
        return;
    }
    const uint32_t a = key_i(key), b = key_j(key);
    const uint32_t L = slot >= 0 ? or_len(slot) : 0u;
    const bool rev = slot >= 0 && or_rev(slot);
    const bool ok = slot < 0 ? (a >= 1 && b < n && b >= a + 2)
                             : (a >= 1 && a + L <= n - 1 &&
                                (b + 2 <= a || (b >= a + L && b + 2 <= n)));
    if (!ok) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            atomicOr(&st->status, kErrBadKey);
            st->converged = 1;
        }
        return;
    }
    OrderedCity* Qs = cur ? T.Q[1] : T.Q[0];
    uint32_t* Rs = cur ? T.route[1] : T.route[0];
    OrderedCity* Qd = cur ? T.Q[0] : T.Q[1];
    uint32_t* Rd = cur ? T.route[0] : T.route[1];
    if (slot < 0)
        gather_tour(Qs, Rs, Qd, Rd, n, T.pos,
                    [=] __device__(uint32_t k) { return rotrev_src(k, a, b, n); });
    else
        gather_tour(Qs, Rs, Qd, Rd, n, T.pos,
                    [=] __device__(uint32_t k) { return oropt_src(k, a, L, b, rev); });
    if (last_block_done(&st->done_blocks)) {
        const unsigned long long m = st->moves;
        if (st->move_log && m < st->log_cap) {
            st->move_log[3 * m + 0] = key_delta(key);
            st->move_log[3 * m + 1] =
                slot < 0 ? (int)a : -1 - (int)(a + ((uint32_t)slot << 21));
            st->move_log[3 * m + 2] = (int)b;
        }
        st->moves = m + 1;
        st->total_moves += 1;
        st->sweeps += 1;
        st->best_key = kNoMove;
        for (int v = 0; v < kOrSlots; ++v) st->or_key[v] = kNoMove;
        st->cur = cur ^ 1;
        if (m + 1 >= st->max_moves) {
            st->converged = 1;
            atomicOr(&st->status, kErrMoveLimit);
        }
    }
}

__global__ void resume_descent_kernel(DevState* st) {
    chain_wait();
    chain_release();
    const unsigned int bad = st->status | st->bad_route;  // includes the move limit
    if (!bad) {
        st->converged = 0u;
        st->best_key = kNoMove;
        for (int v = 0; v < kOrSlots; ++v) st->or_key[v] = kNoMove;
    }
}

cudaError_t launch_resume_descent(const TourBufs& T, cudaStream_t s) {
    return launch_chained(resume_descent_kernel, 1, 1, 0, s, T.st);
}

cudaError_t launch_apply_nbr_move(const TourBufs& T, cudaStream_t s) {
    return launch_chained(apply_nbr_move_kernel, grid_for(T.n), kThreads, 0, s, T);
}

cudaError_t launch_apply_move(const TourBufs& T, cudaStream_t s, uint32_t* out) {
    return launch_chained(apply_move_kernel, grid_for(T.n), kThreads, 0, s, T, out);
}
cudaError_t launch_tour_length(const TourBufs& T, cudaStream_t s) {
    tour_length_kernel<<<grid_for(T.n), kThreads, 0, s>>>(T);
    return cudaGetLastError();
}
cudaError_t launch_kick(const TourBufs& T, int kind, cudaStream_t s) {
    kick_kernel<<<grid_for(T.n), kThreads, 0, s>>>(T, kind);
    return cudaGetLastError();
}
cudaError_t launch_accept(const TourBufs& T, cudaStream_t s) {
    accept_kernel<<<grid_for(T.n), kThreads, 0, s>>>(T);
    return cudaGetLastError();
}
cudaError_t launch_save_best(const TourBufs& T, cudaStream_t s) {
    save_best_kernel<<<grid_for(T.n), kThreads, 0, s>>>(T);
    return cudaGetLastError();
}

}  // namespace logo
