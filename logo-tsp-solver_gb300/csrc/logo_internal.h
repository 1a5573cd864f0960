// Host-side declarations shared by the translation units of liblogo_gpu.so.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/logo_gpu.h"
#include "logo_device.cuh"

namespace logo {

// Programmatic dependent launches for the step chain (see chain_wait in
// logo_device.cuh) when launched on a stream; inside stream capture (the
// descent and ILS graphs, whose launches the graph already pipelines) the
// launches stay ordinary.  Measured on GB300 at n = 100k: a step launched
// on a stream 0.0769 -> 0.0730 ms (the sweep's three launches 0.0642 ->
// 0.0604 ms); captured descents unchanged with the exhaustive search and
// 15 % slower with the neighbour search.  Off when the environment sets
// LOGO_CHAINED_LAUNCH=0.
bool chained_launch_enabled();
template <typename... KArgs, typename... Args>
cudaError_t launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                           cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) cap = cudaStreamCaptureStatusActive;
    cfg.numAttrs = chained_launch_enabled() && cap == cudaStreamCaptureStatusNone ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// ---- single-instance sweep (sweep.cu) ---------------------------------------
struct SweepLaunch {
    const OrderedCity* Q0;
    const OrderedCity* Q1;
    uint32_t n;
    const uint2* tiles;  // (row0, col0) per CTA
    uint32_t ntiles;
    uint32_t cb;         // columns per tile
    int R, NW;           // rows per thread, warps per CTA
    int variant;         // LOGO_SWEEP_* (0 MUFU, 4 fused, 5 local, 6 boxed; 1-3 retired)
    float margin;        // filter margin M
    DevState* st;
    // boxed variant (6): per 32-column window (columns 3 + 32g ..) its coordinate
    // bounding box and largest edge (sweep_windows(n) entries), the same per
    // 32-row window (rows 1 + 32g .., sweep_row_windows(n) entries), the list
    // of (tile, column-window mask) that pass the window test (ntiles entries)
    // and its three counters (tiles listed from the start, claimed, listed from the end)
    float4* wbox;
    float* wmax;
    float4* rbox;
    float* rmax;
    uint4* work;         // ntiles entries
    uint32_t* workctl;   // tiles listed from the start, claimed, listed from the end
    // boxed variant: the tour's city ids (both buffers), the tour position of
    // every city (written by the window pass) and kSeedNeighbours nearest
    // neighbours per city, whose pairs seed the sweep's best delta
    const uint32_t* R0;
    const uint32_t* R1;
    uint32_t* pos;
    const uint32_t* nbr;
};
constexpr uint32_t kSeedNeighbours = 5;
// k nearest other cities of every city, out[v * k + j] (construct.cpp).
void knn_grid(const ::logo_xy* p, uint32_t n, uint32_t k, uint32_t* out);
// Windows of the boxed variant: columns 3 + 32 g .. 3 + 32 g + 31 (< n) and
// rows 1 + 32 g .. 1 + 32 g + 31 (rows with pairs: i + 3 <= n).
__host__ __device__ inline uint32_t sweep_windows(uint32_t n) {
    return n < 4 ? 1 : (n - 3 + 31) / 32;
}
__host__ __device__ inline uint32_t sweep_row_windows(uint32_t n) {
    return n < 4 ? 1 : (n - 3 + 31) / 32;
}
// The boxed variant needs tile widths that are multiples of 32 (tile column
// starts are then 3 + 32k) and at most 1024 (one mask bit per window).
inline bool sweep_cols_supported(int variant, uint32_t cb) {
    return variant != 6 || (cb % 32 == 0 && cb <= 1024);
}
cudaError_t launch_sweep(const SweepLaunch& L, cudaStream_t s);
// Sets the kernel attributes of L's shape; call before any stream capture.
cudaError_t launch_sweep_prepare(const SweepLaunch& L);
bool sweep_shape_supported(int R, int NW, int variant);
size_t sweep_smem_bytes(uint32_t cb);

struct CoopSync;  // coop.cu's grid barrier and key slots (below)

// ---- neighbour-list search (neighbour.cu) ------------------------------------
struct NbrLaunch {
    const OrderedCity* Q0;
    const OrderedCity* Q1;
    const uint32_t* R0;
    const uint32_t* R1;
    OrderedCity* Q0w;     // the same buffers, writable (the cooperative phase moves the tour)
    OrderedCity* Q1w;
    uint32_t* R0w;
    uint32_t* R1w;
    uint32_t* pos;        // tour position of every city (exact: kept by every tour move)
    const uint32_t* nbr;  // K nearest other cities per city, nearest first
    uint32_t K;
    uint32_t n;
    DevState* st;
    bool oropt;           // also the Or-opt candidates (into st->or_key)
    float margin;         // filter_margin of the instance (Or-opt estimate test)
};
// Default and largest neighbour-list length of LOGO_SEARCH_NEIGHBOUR.
constexpr uint32_t kSearchNeighbours = 8, kSearchNeighboursMax = 16;
// One neighbour sweep: the lowest improving candidate key into st->best_key
// (the apply kernel then moves or marks convergence), st->nbr_sweeps += 1.
cudaError_t launch_nbr_sweep(const NbrLaunch& L, cudaStream_t s);
// Recomputes pos from the current tour.
cudaError_t launch_fill_pos(const NbrLaunch& L, cudaStream_t s);
// The whole neighbour phase of a descent as one cooperative launch
// (coop.cu): moves until no candidate improves or st->max_moves; cs must
// hold count = gen = 0 and every slot = kNoMove.  coop_nbr_grid: its CTAs
// for this n (0: cooperative launches unavailable).
int coop_nbr_grid(uint32_t n, bool oropt, int device);
cudaError_t launch_coop_nbr(const NbrLaunch& L, CoopSync* cs, int grid, cudaStream_t s);

// ---- tour maintenance (tour.cu) --------------------------------------------
struct TourBufs {
    OrderedCity* Q[2];
    uint32_t* route[2];
    OrderedCity* Qbest;
    uint32_t* route_best;
    const float2* xy;
    uint32_t n;
    DevState* st;
    uint32_t* seen;  // n words: number of the last route load that met each city
    // tour position of every city (boxed sweep's seed pass; null otherwise),
    // kept current by every kernel that moves the tour
    uint32_t* pos;
};
// Cooperative persistent descent (coop.cu) for tours up to kCoopMaxN cities:
// one launch runs the descent to a local optimum or st->max_moves.
constexpr uint32_t kCoopMaxN = 6144;
struct CoopSync {
    unsigned int count;            // CTAs arrived at the current barrier
    unsigned int gen;              // barrier generation
    unsigned long long slot[3];    // best key of move m in slot m % 3
    unsigned long long or_slot[3][5];  // neighbour phase: Or-opt keys per variant
};
struct CoopArgs {
    OrderedCity* Q0;
    OrderedCity* Q1;
    uint32_t* R0;
    uint32_t* R1;
    uint32_t n;
    float margin;
    DevState* st;
    CoopSync* cs;  // count = gen = 0 and every slot = kNoMove before the launch
    // ILS launch only: coordinates by city id, the best tour (also the start:
    // route_best/Qbest and st->best_length are set before the launch) and the
    // kick count and kind
    const float2* xy;
    OrderedCity* Qbest;
    uint32_t* route_best;
    uint32_t kicks;
    int kick_kind;
};
// CTAs for a cooperative launch at this n on `device` (0: not available);
// coop_ils_grid for the launch that runs a whole ILS call.
int coop_grid(uint32_t n, int device);
int coop_ils_grid(uint32_t n, int device);
cudaError_t launch_coop_descent(const CoopArgs& A, int grid, cudaStream_t s);
// One cooperative launch runs descent, length, accept/revert and kicks for
// A.kicks kicks (ILSGlobalSolverSequential::optimize with a kick count).
cudaError_t launch_coop_ils(const CoopArgs& A, int grid, cudaStream_t s);
// One CTA waits at the cooperative grid barrier sized for two (test hook).
cudaError_t launch_barrier_probe(CoopSync* cs, DevState* st, cudaStream_t s);

// Loads a tour from src (a host buffer the device reads in place, or a
// device copy) into route[0] and Q[0], with pos and the permutation check
// (st->bad_route = 1 if src is not a permutation of 0..n-1; `epoch` must
// differ from every value seen holds, i.e. count loads from 1 with seen
// zeroed at the start and on wrap-around); cur = 0.  With reset_moves != 0
// also what launch_reset_descent(reset_moves) does.
cudaError_t launch_load_route(const TourBufs& T, const uint32_t* src, uint32_t epoch,
                              unsigned long long reset_moves, cudaStream_t s);
// Writes the current tour (best: the ILS best) to dst (host buffer written
// in place, or device memory).
cudaError_t launch_store_route(const TourBufs& T, uint32_t* dst, bool best, cudaStream_t s);
// Prepares *st for a new descent: cur = 0 kept, counters cleared.
cudaError_t launch_reset_descent(const TourBufs& T, unsigned long long max_moves,
                                 cudaStream_t s);
// Applies the move in st->best_key (or marks convergence); with out, also
// writes the resulting current tour there (moved or not).
cudaError_t launch_apply_move(const TourBufs& T, cudaStream_t s, uint32_t* out = nullptr);
// The same for the neighbour search with Or-opt moves: the best of
// st->best_key and st->or_key[].
cudaError_t launch_apply_nbr_move(const TourBufs& T, cudaStream_t s);
// After a converged neighbour phase: continue the same descent (moves and
// limit kept) with full sweeps, unless it stopped on an error or the limit.
cudaError_t launch_resume_descent(const TourBufs& T, cudaStream_t s);
// st->length = length of the current tour.
cudaError_t launch_tour_length(const TourBufs& T, cudaStream_t s);
// ILS pieces.
cudaError_t launch_kick(const TourBufs& T, int kind, cudaStream_t s);
cudaError_t launch_accept(const TourBufs& T, cudaStream_t s);
cudaError_t launch_save_best(const TourBufs& T, cudaStream_t s);
// Kick of the kind in st->kick_kind.
inline cudaError_t launch_kick_dev(const TourBufs& T, cudaStream_t s) { return launch_kick(T, -1, s); }
// Set the WHILE conditions of the device-run ILS graph (see tour.cu).
cudaError_t launch_descent_cond(DevState* st, cudaGraphConditionalHandle h, bool first,
                                cudaStream_t s);
cudaError_t launch_kick_cond(DevState* st, cudaGraphConditionalHandle h, bool first,
                             cudaStream_t s);

// Upper bound of |exact delta - approximate delta| for coordinates whose
// bounding-box diagonal is `diag` (see filter_margin in capi.cu).
float filter_margin(double diag);

}  // namespace logo
