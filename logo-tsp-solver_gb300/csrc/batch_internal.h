// Host/device interface of the batched persistent solver (batch.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace logo {

constexpr int kStartGiven = 0, kStartNN = 1, kStartMF = 2;

constexpr uint32_t kBatchMaxN = 4096;  // largest instance a CTA holds in smem

constexpr uint32_t kNoGroup = 0xFFFFFFFFu;

struct BatchInstance {
    unsigned long long off;   // first city of this instance in coords / routes
    unsigned long long seed;  // kick PRNG state
    uint32_t n;
    float margin;             // filter margin for this instance's coordinates
    uint32_t group;           // shared-best group (multi-start), or kNoGroup
    uint32_t pad;
};

// Best tour shared by the replicas of one multi-start group.  A writer holds
// `lock` (taken with atomicCAS, never waited for) and makes `seq` odd while
// it rewrites the tour; a reader keeps a copy only if `seq` was even and
// unchanged around it.
struct SharedBest {
    unsigned long long best_len;  // ~0 until the first publication
    unsigned int lock;
    unsigned int seq;
    unsigned long long off;       // the tour's first entry in BatchArgs::shared_tours
};

struct BatchResult {
    unsigned long long start_length;
    unsigned long long best_length;
    unsigned long long moves;
    unsigned long long sweeps;
    uint32_t kicks;
    uint32_t accepted;
    uint32_t status;          // kErr* bits
    uint32_t pad;
};

struct BatchArgs {
    const float2* coords;     // all instances' coordinates, concatenated
    uint32_t* routes;         // start tours in, best tours out
    const BatchInstance* inst;
    const uint32_t* order;    // queue order (instances by descending n)
    BatchResult* results;
    unsigned int* queue;      // next slot of `order` to hand out
    uint32_t count;
    uint32_t max_n;           // sizes the dynamic shared memory
    uint32_t kicks;
    int kick_kind;
    SharedBest* shared;       // per group (null when no instance has a group)
    uint32_t* shared_tours;   // the groups' best tours
    int start;                // kStartGiven, or kStartNN: build nearest-neighbour tours instead of loading them
};

struct BatchShape {
    int R;   // rows per thread
    int NT;  // threads per CTA
    int TC;  // columns per warp tile
};

size_t batch_smem_bytes(uint32_t max_n);
// Launches the persistent kernel with `grid` CTAs; with occupancy != null
// only reports CTAs per SM for this shape and max_n.
// Multiple-fragment start tours of instances order[0 .. count) written into
// routes (equal to logo_mf_tour), one CTA per instance at a time;
// prepare_mf_start (outside any stream capture) raises the kernel's shared
// memory limit first.
cudaError_t prepare_mf_start();
// One instance's nearest-neighbour (kStartNN) or multiple-fragment
// (kStartMF) start tour into route (device memory), n <= kBatchMaxN.
cudaError_t launch_start_tour(const float2* xy, uint32_t n, int kind, uint32_t* route,
                              cudaStream_t s);
cudaError_t launch_mf_start(const float2* coords, uint32_t* routes, const BatchInstance* inst,
                            const uint32_t* order, uint32_t count, uint32_t max_n, int sms,
                            cudaStream_t s);
cudaError_t launch_batch(const BatchArgs& A, const BatchShape& sh, int grid, cudaStream_t s,
                         int* occupancy);
// Lists the compiled shapes; returns how many there are.
int batch_shapes(BatchShape* out, int cap);

}  // namespace logo
