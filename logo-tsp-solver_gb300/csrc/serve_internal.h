// Host/device interface of the serving rounds (serve.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace logo {

constexpr uint32_t kServeInit = 0, kServeDescent = 1, kServeAccept = 2, kServeDone = 3;

// Device-resident state of one admitted request (one slot).
struct ServeSlot {
    unsigned long long off;           // first city of the slot in the arena
    unsigned long long rng;           // kick PRNG state
    unsigned long long start_len;
    unsigned long long best_len;
    unsigned long long moves;
    unsigned long long sweeps;
    unsigned long long descent_moves; // moves of the current descent
    uint32_t n;
    uint32_t phase;                   // kServe*
    uint32_t kicks_done;
    uint32_t kicks_total;
    uint32_t accepted;
    uint32_t status;                  // kErr* bits
    int kick_kind;
    float margin;
};

struct ServeArgs {
    const float2* coords;  // arena: coordinates by city id, per slot
    uint32_t* route;       // arena: current tours
    uint32_t* best;        // arena: best tours
    ServeSlot* slots;
    const uint32_t* units; // slots to advance this round
    uint32_t nunits;
    unsigned int* queue;   // next unit to hand out
    uint32_t max_n;        // sizes the dynamic shared memory
    unsigned long long budget_pairs;
};

size_t serve_smem_bytes(uint32_t max_n);
cudaError_t launch_serve_round(const ServeArgs& A, int grid, cudaStream_t s, int* occupancy);

}  // namespace logo
