// Device-side building blocks shared by the 2-opt kernels (sm_103a).
//
// Distances.  The reference's per-edge distance is
//     (int)(sqrtf(dx*dx + dy*dy) + 0.5f)          src/cuda/cuda_common.h:33-40
// Its kernels are built with --use_fast_math (Makefile:84), its CPU length
// with the C compiler's default contraction; this library fixes the
// arithmetic to IEEE binary32 with no FMA contraction and a correctly rounded
// square root, so the CPU oracle and the device agree bit for bit
// (exact_dist).
//
// The sweeps do not evaluate exact_dist for every pair.  The MUFU screen
// evaluates approx_dist (one MUFU sqrt) for every pair and a conservative
// error bound M (host-side filter_margin) tells it which pairs could still
// tie or beat the best exact delta it has seen; only those are re-evaluated
// exactly (the other screens use proven bounds on squared distances and
// bounding boxes instead of M).  A pair whose exact delta is <= the bound
// always passes the filter, so the chosen move is the exact lowest-(delta,
// i, j) one.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace logo {

constexpr uint64_t kNoMove = ~0ull;
constexpr int kKeyDeltaBias = 1 << 22;  // delta in [-2^22, 0)
constexpr uint32_t kMaxCities = 1u << 21;  // MAX_CITIES, src/defs.h:25

// Error bits of DevState::status.
constexpr uint32_t kErrTimeout = 1u;     // a bounded wait ran out
constexpr uint32_t kErrMoveLimit = 2u;   // descent hit its move limit
constexpr uint32_t kErrBadKey = 4u;      // a key decoded outside [0, n)
constexpr uint32_t kErrInternal = 8u;

// Tour-ordered city record: position k of the tour holds city route[k] at
// (x, y); e is the exact length of the edge entering k, i.e.
// d(k-1, k) for k >= 1 and the closing edge d(n-1, 0) for k = 0.
struct __align__(16) OrderedCity {
    float x, y, e, pad;
};

// Device-resident control block of one single-instance solve.
struct DevState {
    unsigned long long best_key;    // argmin of the current sweep
    unsigned long long moves;       // moves applied in this descent
    unsigned long long total_moves; // moves over the whole call (ILS)
    unsigned long long sweeps;
    unsigned long long max_moves;
    unsigned long long rng;         // SplitMix64 state for kicks
    unsigned long long length;      // tour length from tour_length_kernel
    unsigned long long best_length; // ILS best
    unsigned long long accepted;
    unsigned long long kicks;
    unsigned long long sweeps_at_reset;  // sweeps when the current descent began
    unsigned int cur;               // which buffer holds the tour
    unsigned int converged;
    unsigned int status;            // kErr* bits
    unsigned int done_blocks;       // last-block-done counter
    unsigned int log_cap;
    unsigned int len_done;          // last-block counter of the length sum
    unsigned int bad_route;         // the last loaded route is not a permutation
    int* move_log;                  // (delta, i, j) per move, or null
    unsigned long long length_acc;  // partial sums of tour_length_kernel
    // ILS run on the device (one graph or one cooperative launch per call)
    unsigned long long kick_target; // kicks to apply in this call
    unsigned long long loop_mark;   // moves at the previous descent-loop check
    unsigned long long ils_iters;   // kick-loop passes so far (guard)
    unsigned long long start_length; // length of the tour the call started from
    unsigned int kick_kind;         // LOGO_KICK_SEGMENT or LOGO_KICK_DOUBLE_BRIDGE
    unsigned int load_bad;          // set by a CTA of load_route_kernel that met a bad id
    unsigned long long nbr_sweeps;  // neighbour sweeps of this descent (or ILS call)
    unsigned long long or_key[5];   // best Or-opt candidate per variant (see or_slot)
};

__host__ __device__ __forceinline__ uint64_t pack_key(int delta, uint32_t i,
                                                      uint32_t j) {
    return ((uint64_t)(uint32_t)(delta + kKeyDeltaBias) << 42) |
           ((uint64_t)i << 21) | (uint64_t)j;
}
__host__ __device__ __forceinline__ int key_delta(uint64_t k) {
    return (int)(k >> 42) - kKeyDeltaBias;
}
__host__ __device__ __forceinline__ uint32_t key_i(uint64_t k) {
    return (uint32_t)((k >> 21) & 0x1FFFFF);
}
__host__ __device__ __forceinline__ uint32_t key_j(uint64_t k) {
    return (uint32_t)(k & 0x1FFFFF);
}

// Canonical per-edge EUC_2D nint distance: IEEE binary32, no contraction,
// correctly rounded sqrt, +0.5f rounded to nearest, truncation toward zero.
__device__ __forceinline__ int exact_dist(float ax, float ay, float bx,
                                          float by) {
    float dx = __fsub_rn(ax, bx);
    float dy = __fsub_rn(ay, by);
    float s = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    return __float2int_rz(__fadd_rn(__fsqrt_rn(s), 0.5f));
}

// Approximate Euclidean distance for the filter: contracted sum of squares
// and the hardware square-root approximation (one MUFU operation).
__device__ __forceinline__ float approx_dist(float ax, float ay, float bx,
                                             float by) {
    float dx = ax - bx;
    float dy = ay - by;
    float s = __fmaf_rn(dy, dy, dx * dx);
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s));
    return r;
}

// SplitMix64 (Steele, Lea, Flood 2014), identical to the oracle's.
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint32_t uniform_below(uint64_t& s,
                                                           uint32_t n) {
    uint64_t hi = splitmix64(s) >> 32;
    return (uint32_t)((hi * (uint64_t)n) >> 32);
}

// Source position of new position k after "rotate by p, reverse [q-p, n)"
// (src/solvers/twoOptLocalSolver.cpp:41-48 and the kick,
// src/solvers/ILSGlobalSolver.cpp:37-48), p <= q.
__host__ __device__ __forceinline__ uint32_t rotrev_src(uint32_t k, uint32_t p,
                                                        uint32_t q,
                                                        uint32_t n) {
    if (k < q - p) return k + p;
    uint32_t s = q + n - 1 - k;  // < 2n
    return s >= n ? s - n : s;
}

// Source position of new position k after a double bridge with cuts
// p1 <= p2 <= p3: old[0,p1) old[p2,p3) old[p1,p2) old[p3,n).
__host__ __device__ __forceinline__ uint32_t bridge_src(uint32_t k, uint32_t p1,
                                                        uint32_t p2,
                                                        uint32_t p3) {
    if (k < p1) return k;
    uint32_t l2 = p3 - p2;
    if (k < p1 + l2) return p2 + (k - p1);
    if (k < p3) return p1 + (k - p1 - l2);
    return k;
}

// ---- Or-opt moves of the neighbour search -------------------------------------
// Segment [s, s+L) (L = 1..3, 1 <= s, s+L <= n-1) moved into the gap after
// old position p (p + 1 <= s - 1, or s + L <= p <= n - 2), in tour order
// (forward) or reversed.  Variants in tie order: slot 0 = L1, 1 = L2, 2 = L2
// reversed, 3 = L3, 4 = L3 reversed; each slot keeps pack_key(delta, s, p).
constexpr int kOrSlots = 5;
__host__ __device__ __forceinline__ int or_slot(uint32_t L, bool rev) {
    return L == 1 ? 0 : (int)(2 * L - 3) + (rev ? 1 : 0);
}
__host__ __device__ __forceinline__ uint32_t or_len(int slot) {
    return slot == 0 ? 1u : (uint32_t)((slot + 3) / 2);
}
__host__ __device__ __forceinline__ bool or_rev(int slot) { return slot == 2 || slot == 4; }
// Source position of new position k after the Or-opt move (s, L, p, rev).
__host__ __device__ __forceinline__ uint32_t oropt_src(uint32_t k, uint32_t s, uint32_t L,
                                                       uint32_t p, bool rev) {
    if (p >= s + L) {  // the segment moves right: old[0,s) old[s+L,p] seg old[p+1,n)
        if (k < s || k > p) return k;
        if (k < p + 1 - L) return k + L;
        const uint32_t t = k - (p + 1 - L);
        return rev ? s + L - 1 - t : s + t;
    }
    // the segment moves left: old[0,p] seg old[p+1,s) old[s+L,n)
    if (k <= p || k >= s + L) return k;
    if (k < p + 1 + L) {
        const uint32_t t = k - (p + 1);
        return rev ? s + L - 1 - t : s + t;
    }
    return k - L;
}

// ---- programmatic dependent launch -------------------------------------------
// Kernels of the step chain (route load, sweeps, move, route store) are
// launched with programmatic stream serialization (launch_chained in
// logo_internal.h): a kernel may be scheduled while the previous one drains.
// Each calls chain_wait() before touching memory -- it returns once the
// previous kernel has completed and its writes are visible, and is a no-op
// for an ordinary launch -- and chain_release() right after, which lets the
// next kernel of the chain be scheduled.  Because every CTA waits before it
// can finish, a kernel completes only after its predecessor did, so the
// chain stays ordered end to end.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void chain_release() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---- warp / block reductions ----------------------------------------------
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- bounded waits ----------------------------------------------------------
// Every spin in this library is bounded by %globaltimer: past the budget the
// waiter records kErrTimeout in the status word and gives up.
__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
constexpr uint64_t kWaitBudgetNs = 2000000000ull;  // 2 s

// ---- mbarrier + bulk copy (TMA, non-tensor form) ----------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(count));
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's earlier shared-memory accesses (and, after a CTA
// barrier, the CTA's) before later bulk-copy (async proxy) writes to them.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar,
                                                      uint32_t bytes) {
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_u32(bar)),
        "r"(bytes)
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bulk global->shared copy completing on `bar`.  dst, src 16-byte aligned;
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// Waits for phase `parity` of `bar`; false (and kErrTimeout in *status)
// if it did not complete within kWaitBudgetNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar,
                                                  uint32_t parity,
                                                  unsigned int* status) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 0; it < (1u << 30); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63) == 63 && global_timer_ns() - t0 > kWaitBudgetNs) break;
    }
    atomicOr(status, kErrTimeout);
    return false;
}

}  // namespace logo
