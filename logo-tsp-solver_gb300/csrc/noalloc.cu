// logo_best_move_noalloc: the best-improvement sweep for callers that must not
// allocate device memory.
//
// Who needs it: callers that account for every device byte in their own pool
// allocator (a framework's caching allocator, a budgeted multi-tenant
// service), and latency-sensitive callers for whom cudaMalloc/cudaFree are off
// limits because those calls can synchronize the whole device.  Such a caller
// allocates the inputs and the output itself and passes device pointers; this
// entry point then launches four kernels on the caller's stream and performs
// no allocation of any kind.
//
// Its working memory (the tour-ordered cities, the argmin key, the bounding
// box and a status word) lives in one file-scope __device__ array of fixed
// size, logo_noalloc_scratch, sized for LOGO_NOALLOC_MAX_CITIES cities
// (1 MiB plus an 8.25 KiB header).  The array exists once per GPU that loads
// the library and stays allocated until the process exits.  Host code cannot
// use the array's name as a device address, so the first call on each device
// looks the address up with cudaGetSymbolAddress (with that device current)
// and caches it; make that first call before any stream capture.  The cache
// is keyed by the device's current context (its driver-assigned unique id),
// so a call after cudaDeviceReset, which re-creates the primary context and
// with it the array, looks the address up again instead of using the old
// one.
//
// The coordinates are read as 8-byte (x, y) pairs, so coords must be 8-byte
// aligned (any cudaMalloc'd array and any even element offset into one);
// route, out and status_out must be 4-byte aligned.  Misaligned pointers are
// refused on the host with LOGO_ERR_INVALID_ARG before any work is enqueued.
//
// Every call shares the array and the array keeps the previous call's
// contents: each call clears the key, bounding box and status first.  Calls
// whose kernels overlap on the GPU (different streams, or different host
// threads on the same device) race on the array and must be serialised by
// the caller.
#include <cmath>
#include <cstdint>
#include <mutex>

#include <cudaTypedefs.h>

#include "../../include/logo_gpu.h"
#include "logo_device.cuh"
#include "sweep_core.cuh"

namespace {

using namespace logo;

constexpr uint32_t kNoAllocMax = LOGO_NOALLOC_MAX_CITIES;

struct __align__(256) NoAllocHeader {
    unsigned long long key;  // argmin of this call
    unsigned int bbox[4];    // min x, min y, max x, max y as ordered integers
    unsigned int status;     // 0, or LOGO_ERR_INVALID_ARG
    unsigned int seen[kNoAllocMax / 32];  // one bit per city id: permutation check
};

constexpr size_t kScratchBytes =
    sizeof(NoAllocHeader) + sizeof(OrderedCity) * (size_t)kNoAllocMax;

static __device__ __align__(256) unsigned char logo_noalloc_scratch[kScratchBytes];

// float <-> integer whose unsigned order matches the float order
__device__ __forceinline__ unsigned int ordered_bits(float f) {
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_ordered(unsigned int o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

__global__ void noalloc_reset(unsigned char* scratch) {
    NoAllocHeader* h = reinterpret_cast<NoAllocHeader*>(scratch);
    for (uint32_t w = threadIdx.x; w < kNoAllocMax / 32; w += blockDim.x) h->seen[w] = 0u;
    if (threadIdx.x == 0) {
        h->key = kNoMove;
        h->bbox[0] = 0xFFFFFFFFu;
        h->bbox[1] = 0xFFFFFFFFu;
        h->bbox[2] = 0u;
        h->bbox[3] = 0u;
        h->status = 0u;
    }
}

// Tour-ordered cities with exact incoming edges; bounding box; route and
// coordinate checks (out-of-range or repeated ids and non-finite coordinates
// set the status word; out-of-range ids are clamped so no access leaves the
// caller's arrays).
__global__ void noalloc_prepare(const float2* __restrict__ xy, const uint32_t* __restrict__ route,
                                uint32_t n, unsigned char* scratch) {
    NoAllocHeader* h = reinterpret_cast<NoAllocHeader*>(scratch);
    OrderedCity* Q = reinterpret_cast<OrderedCity*>(scratch + sizeof(NoAllocHeader));
    unsigned int mnx = 0xFFFFFFFFu, mny = 0xFFFFFFFFu, mxx = 0u, mxy = 0u;
    bool bad = false;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        uint32_t c = route[k], p = route[k == 0 ? n - 1 : k - 1];
        if (c >= n || p >= n) {
            bad = true;
            c = c < n ? c : 0;
            p = p < n ? p : 0;
        } else if (atomicOr(&h->seen[c >> 5], 1u << (c & 31)) & (1u << (c & 31))) {
            bad = true;  // a repeated city id: not a permutation
        }
        const float2 a = xy[c], b = xy[p];
        if (!isfinite(a.x) || !isfinite(a.y)) bad = true;
        OrderedCity o;
        o.x = a.x;
        o.y = a.y;
        o.e = (float)exact_dist(b.x, b.y, a.x, a.y);
        o.pad = 0.f;
        Q[k] = o;
        mnx = min(mnx, ordered_bits(a.x));
        mny = min(mny, ordered_bits(a.y));
        mxx = max(mxx, ordered_bits(a.x));
        mxy = max(mxy, ordered_bits(a.y));
    }
    atomicMin(&h->bbox[0], mnx);
    atomicMin(&h->bbox[1], mny);
    atomicMax(&h->bbox[2], mxx);
    atomicMax(&h->bbox[3], mxy);
    if (bad) atomicExch(&h->status, (unsigned int)LOGO_ERR_INVALID_ARG);
}

// Same exactness margin as the library's other sweeps, from the box diagonal.
__device__ __forceinline__ float noalloc_margin(double diag) {
    const double rel = 9.5367431640625e-07;  // 2^-20
    const double u = 5.9604644775390625e-08;  // 2^-24
    return (float)(1.0 + 2.0 * diag * (3.0 * u + rel) + 2.0 * 1.1920928955078125e-07 +
                   3.0 * u * 4.0 * diag + 1.0);
}

constexpr int kR = 4;
constexpr int kNW = 4;
constexpr uint32_t kRowsPerCta = 32u * kR * kNW;  // 512
constexpr uint32_t kColsPerCta = 256;

// grid (column chunk, row block); tiles entirely below the diagonal exit.
__global__ void __launch_bounds__(kNW * 32)
    noalloc_sweep(uint32_t n, unsigned char* scratch) {
    NoAllocHeader* h = reinterpret_cast<NoAllocHeader*>(scratch);
    const OrderedCity* Q = reinterpret_cast<const OrderedCity*>(scratch + sizeof(NoAllocHeader));
    __shared__ unsigned long long wbest[kNW];
    const uint32_t row0 = 1 + blockIdx.y * kRowsPerCta;
    const uint32_t col0 = 3 + blockIdx.x * kColsPerCta;
    if (row0 + 3 > n || col0 > n - 1 || col0 + kColsPerCta <= row0 + 2) return;
    if (*(volatile unsigned int*)&h->status) return;
    const double dx = (double)from_ordered(h->bbox[2]) - (double)from_ordered(h->bbox[0]);
    const double dy = (double)from_ordered(h->bbox[3]) - (double)from_ordered(h->bbox[1]);
    const double diag = sqrt(dx * dx + dy * dy);
    if (!(diag < LOGO_MAX_DIAGONAL)) {
        if (threadIdx.x == 0) atomicExch(&h->status, (unsigned int)LOGO_ERR_INVALID_ARG);
        return;
    }
    const float margin = noalloc_margin(diag);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ib = row0 + (warp * 32 + lane) * kR;
    uint64_t best = kNoMove;
    int B = -1;
    RowBlock<kR> rb;
    load_rows<kR>(rb, Q, ib, n);
    refresh_thresholds<kR>(rb, Q, ib, n, B, margin);
    walk_columns<kR>(rb, Q, 0, col0, min(col0 + kColsPerCta, n), ib, n, Q, margin, B, best);
    best = warp_min_u64(best);
    if (lane == 0) wbest[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = wbest[0];
        for (int w = 1; w < kNW; ++w) m = wbest[w] < m ? wbest[w] : m;
        if (m != kNoMove) atomicMin(&h->key, m);
    }
}

__global__ void noalloc_finish(const unsigned char* scratch, logo_move* out, int32_t* status_out) {
    const NoAllocHeader* h = reinterpret_cast<const NoAllocHeader*>(scratch);
    const unsigned long long k = h->key;
    logo_move m;
    if (h->status || k == kNoMove) {
        m.i = 0;
        m.j = 0;
        m.minchange = 0;
    } else {
        m.i = key_i(k);
        m.j = key_j(k);
        m.minchange = key_delta(k);
    }
    *out = m;
    if (status_out) *status_out = (int32_t)h->status;
}

// The scratch array's device address per device, with the id of the context
// it was looked up in (0: not looked up yet).
struct ScratchAddr {
    unsigned long long ctx_id;
    void* ptr;
};
std::mutex g_mu;
ScratchAddr g_scratch[64] = {};
PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_id = nullptr;
bool g_ctx_fns_tried = false;

// Unique id of the calling thread's current context; 0 if the driver cannot
// tell, in which case the address is looked up on every call.
unsigned long long current_ctx_id() {
    if (!g_ctx_fns_tried) {
        g_ctx_fns_tried = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault,
                                             &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault,
                                             &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            g_ctx_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f1);
            g_ctx_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f2);
        }
    }
    if (!g_ctx_current || !g_ctx_id) return 0ull;
    CUcontext ctx = nullptr;
    unsigned long long id = 0ull;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return 0ull;
    if (g_ctx_id(ctx, &id) != CUDA_SUCCESS) return 0ull;
    return id;
}

}  // namespace

extern "C" logo_status logo_best_move_noalloc(const logo_xy* coords, const uint32_t* route,
                                              uint32_t n, logo_move* out, int32_t* status_out,
                                              void* stream) {
    if (!coords || !route || !out) return LOGO_ERR_INVALID_ARG;
    if (n < 3 || n > kNoAllocMax) return LOGO_ERR_INVALID_ARG;
    if ((reinterpret_cast<uintptr_t>(coords) & 7u) || (reinterpret_cast<uintptr_t>(route) & 3u) ||
        (reinterpret_cast<uintptr_t>(out) & 3u) || (reinterpret_cast<uintptr_t>(status_out) & 3u))
        return LOGO_ERR_INVALID_ARG;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return LOGO_ERR_NO_DEVICE;
    if (dev >= 64) return LOGO_ERR_INVALID_ARG;
    void* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        const unsigned long long id = current_ctx_id();
        ScratchAddr& a = g_scratch[dev];
        if (!a.ptr || id == 0ull || a.ctx_id != id) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, logo_noalloc_scratch) != cudaSuccess || !p)
                return LOGO_ERR_CUDA;
            a.ptr = p;
            a.ctx_id = id;
        }
        scratch = a.ptr;
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* sc = static_cast<unsigned char*>(scratch);
    noalloc_reset<<<1, 256, 0, s>>>(sc);
    const unsigned prep_grid = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    noalloc_prepare<<<prep_grid, 256, 0, s>>>(reinterpret_cast<const float2*>(coords), route, n,
                                              sc);
    if (n >= 4) {
        const dim3 grid((n - 3 + kColsPerCta - 1) / kColsPerCta,
                        (n - 3 + kRowsPerCta - 1) / kRowsPerCta);
        noalloc_sweep<<<grid, kNW * 32, 0, s>>>(n, sc);
    }
    noalloc_finish<<<1, 1, 0, s>>>(sc, out, status_out);
    return cudaGetLastError() == cudaSuccess ? LOGO_OK : LOGO_ERR_CUDA;
}
