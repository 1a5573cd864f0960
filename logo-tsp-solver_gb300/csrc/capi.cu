// C ABI of the single-instance engine (include/logo_gpu.h).
//
// Host side of the path the reference runs in CUDASolver + TwoOptLocalSolver +
// ILSGlobalSolverSequential.  The reference crosses the host/device boundary
// three times per move (gather + H2D of the ordered coordinates, launch, D2H
// of best2_out; src/solvers/CUDASolver.cpp:285-386) and applies the move and
// measures the tour on the host (twoOptLocalSolver.cpp:41-50).  Here the tour
// stays in HBM: a descent is a CUDA graph of `graph_steps` (sweep, apply)
// pairs replayed until the device-side convergence flag is set; the host
// reads one small status block per replay.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/logo_gpu.h"
#include "batch_internal.h"
#include "logo_device.cuh"
#include "logo_internal.h"

using namespace logo;

struct logo_ctx {
    int device = 0;
    uint32_t n = 0;
    cudaStream_t stream = nullptr;
    float2* d_xy = nullptr;
    OrderedCity* d_Q[2] = {nullptr, nullptr};
    uint32_t* d_route[2] = {nullptr, nullptr};
    OrderedCity* d_Qbest = nullptr;
    uint32_t* d_route_best = nullptr;
    DevState* d_st = nullptr;
    DevState* h_st = nullptr;  // pinned mirror
    uint32_t* d_seen = nullptr;   // route permutation check: last load that met each city
    uint32_t load_epoch = 0;      // loads so far (mod 2^32 - 1, from 1)
    int route_io = LOGO_ROUTE_IO_AUTO;
    int search = LOGO_SEARCH_EXHAUSTIVE;
    uint32_t search_k = kSearchNeighbours;  // neighbour-list length of LOGO_SEARCH_NEIGHBOUR
    uint32_t* d_nbr_search = nullptr;       // search_k nearest cities per city
    uint32_t nbr_list_k = 0;                // length d_nbr_search was built with
    cudaGraphExec_t nbr_chunk_exec = nullptr;  // nbr_chunk_steps x (neighbour sweep, apply)
    uint32_t nbr_chunk_steps = 32;
    int nbr_coop_grid = 0;        // CTAs of the cooperative neighbour phase (0: graphs)
    uint32_t* d_start = nullptr;  // logo_start_tour's device output
    bool pageable_ok = false;     // the device reads and writes pageable host memory
    float4* d_wbox = nullptr;     // per-window boxes and largest edges (boxed sweep)
    float* d_wmax = nullptr;
    float4* d_rbox = nullptr;
    float* d_rmax = nullptr;
    uint4* d_work = nullptr;      // boxed sweep: tiles that pass the window test
    uint32_t* d_workctl = nullptr;
    uint32_t* d_pos = nullptr;    // boxed sweep: tour position of every city
    uint32_t* d_nbr = nullptr;    // boxed sweep: kSeedNeighbours nearest cities per city
    CoopSync* d_coop = nullptr;   // barrier and best-key slots of the cooperative descent
    int coop_grid = 0;            // CTAs of the cooperative descent (0: unavailable)
    int coop_ils_grid = 0;        // CTAs of the cooperative ILS launch (0: unavailable)
    int descent_mode = LOGO_DESCENT_AUTO;
    uint2* d_tiles = nullptr;
    uint32_t ntiles = 0;
    int R = 8, NW = 4;
    uint32_t cb = 1024;
    int variant = LOGO_SWEEP_MUFU;
    float margin = 0.f;
    double diag = 0.0;
    cudaGraphExec_t chunk_exec = nullptr;
    cudaGraphExec_t ils_exec = nullptr;  // device-run ILS (graph descent path), built on first use
    uint32_t chunk_steps = 8;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool have_route = false;
    uint64_t host_waits = 0;      // stream/event synchronisations made for this context
    bool poisoned = false;        // a device-side wait timed out: the context is not used again
    std::string err;
};

namespace {

thread_local std::string g_create_err;

const char* kVersion = "logo-gb300 0.1 (sm_103a)";

logo_status fail(logo_ctx* c, logo_status s, const std::string& msg) {
    if (c)
        c->err = msg;
    else
        g_create_err = msg;
    return s;
}

#define CK(ctx, call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? LOGO_ERR_OOM         \
                                                             : LOGO_ERR_CUDA,      \
                        std::string(#call) + ": " + cudaGetErrorString(e_));        \
    } while (0)

TourBufs bufs(const logo_ctx* c) {
    TourBufs T;
    T.Q[0] = c->d_Q[0];
    T.Q[1] = c->d_Q[1];
    T.route[0] = c->d_route[0];
    T.route[1] = c->d_route[1];
    T.Qbest = c->d_Qbest;
    T.route_best = c->d_route_best;
    T.xy = c->d_xy;
    T.n = c->n;
    T.st = c->d_st;
    T.seen = c->d_seen;
    T.pos = c->d_pos;
    return T;
}

NbrLaunch nbr_args(const logo_ctx* c) {
    NbrLaunch L;
    L.Q0 = c->d_Q[0];
    L.Q1 = c->d_Q[1];
    L.R0 = c->d_route[0];
    L.R1 = c->d_route[1];
    L.Q0w = c->d_Q[0];
    L.Q1w = c->d_Q[1];
    L.R0w = c->d_route[0];
    L.R1w = c->d_route[1];
    L.pos = c->d_pos;
    L.nbr = c->d_nbr_search;
    L.K = c->search_k;
    L.n = c->n;
    L.st = c->d_st;
    L.oropt = c->search == LOGO_SEARCH_NEIGHBOUR_OROPT;
    L.margin = c->margin;
    return L;
}

// The move step after a neighbour sweep: with Or-opt candidates the apply
// kernel that also reads their slots.
cudaError_t launch_nbr_apply(const logo_ctx* c, const TourBufs& T, cudaStream_t s) {
    return c->search == LOGO_SEARCH_NEIGHBOUR_OROPT ? launch_apply_nbr_move(T, s)
                                                    : launch_apply_move(T, s);
}

SweepLaunch sweep_args(const logo_ctx* c) {
    SweepLaunch L;
    L.Q0 = c->d_Q[0];
    L.Q1 = c->d_Q[1];
    L.n = c->n;
    L.tiles = c->d_tiles;
    L.ntiles = c->ntiles;
    L.cb = c->cb;
    L.R = c->R;
    L.NW = c->NW;
    L.variant = c->variant;
    L.margin = c->margin;
    L.st = c->d_st;
    L.wbox = c->d_wbox;
    L.wmax = c->d_wmax;
    L.rbox = c->d_rbox;
    L.rmax = c->d_rmax;
    L.work = c->d_work;
    L.workctl = c->d_workctl;
    L.R0 = c->d_route[0];
    L.R1 = c->d_route[1];
    L.pos = c->d_pos;
    L.nbr = c->d_nbr;
    return L;
}

uint64_t pairs_of(uint32_t n) { return n < 4 ? 0 : (uint64_t)(n - 2) * (n - 3) / 2; }

// Pairs decided by `sweeps` sweeps of which `nbr` were neighbour sweeps
// (2K candidate 2-opt pairs per position, and 10K Or-opt candidates with
// LOGO_SEARCH_NEIGHBOUR_OROPT).
uint64_t pair_evals_of(const logo_ctx* c, uint64_t sweeps, uint64_t nbr) {
    nbr = std::min(nbr, sweeps);
    const uint64_t per = (c->search == LOGO_SEARCH_NEIGHBOUR_OROPT ? 12ull : 2ull) * c->search_k;
    return (sweeps - nbr) * pairs_of(c->n) + nbr * per * c->n;
}

// Default tile shape by size (overridable through logo_ctx_set_shape and
// logo_ctx_set_kernel).
void default_shape(uint32_t n, int& R, int& NW, uint32_t& cb, int& variant) {
    // measured on GB300 (one sweep: NN start tours of Gaussian mixtures, the
    // local optimum of the n = 100k one, uniform points on random tours): from
    // n = 17.5k up the boxed screen is fastest (n = 100k NN tour: 0.084 ms with
    // (4, 4, 128) tiles vs 0.61 local, 0.83 fused, 1.80 MUFU; at its local
    // optimum 0.102 vs 0.68; random tour 0.39 vs 0.68, 0.23 with (8, 8, 1024)
    // tiles; n = 40k: 0.063 ms with 64-column tiles vs 0.073 with 128 and
    // 0.149 local; n = 20k: 0.067 vs 0.067 local and 0.084 MUFU; n = 1M random
    // tour: 6.0 ms with (8, 8, 1024) vs 54.8 local); below it the MUFU screen,
    // whose test is tighter on short tours, wins, with 64-column tiles from 3k
    // (n = 10k: 0.030 ms vs 0.063 boxed and 0.042 with (4, 4, 128) MUFU tiles).
    variant = LOGO_SWEEP_MUFU;
    if (n >= 300000) {
        variant = LOGO_SWEEP_BOXED;
        R = 8; NW = 8; cb = 1024;
    } else if (n >= 200000) {
        variant = LOGO_SWEEP_BOXED;
        R = 4; NW = 4; cb = 512;
    } else if (n >= 50000) {
        // with the seeded bound, 64-column tiles (n = 100k descent from the NN
        // tour: 1.37 s against 1.47 s with 128, 1.41 with 32; sweep of the
        // benchmark's states 0.074 ms against 0.080)
        variant = LOGO_SWEEP_BOXED;
        R = 4; NW = 4; cb = 64;
    } else if (n >= 17500) {
        variant = LOGO_SWEEP_BOXED;
        R = 4; NW = 4; cb = 64;
    } else if (n >= 3000) {
        R = 4; NW = 2; cb = 64;
    } else {
        R = 2; NW = 2; cb = 64;
    }
}

// Tiles of the pair triangle: rows [row0, row0 + NW*32*R) x columns
// [col0, col0 + cb); full tiles first, diagonal tiles last.
std::vector<uint2> make_tiles(uint32_t n, int R, int NW, uint32_t cb) {
    std::vector<uint2> full, diag;
    if (n < 4) return full;
    const uint32_t rt = (uint32_t)(NW * 32 * R);
    for (uint32_t row0 = 1; row0 + 3 <= n; row0 += rt) {
        const uint32_t row_last = std::min(row0 + rt - 1, n - 3);
        for (uint32_t col0 = row0 + 2; col0 <= n - 1; col0 += cb) {
            uint2 t = make_uint2(row0, col0);
            if (col0 >= row_last + 2)
                full.push_back(t);
            else
                diag.push_back(t);
        }
    }
    full.insert(full.end(), diag.begin(), diag.end());
    return full;
}

uint32_t pick_graph_steps(uint32_t n) {
    // aim at a few milliseconds of device work per graph launch
    const double step_us = (double)pairs_of(n) / 3.0e6 + 6.0;
    double s = 4000.0 / step_us;
    if (s < 4) s = 4;
    if (s > 256) s = 256;
    return (uint32_t)s;
}

logo_status rebuild(logo_ctx* c) {
    if (c->chunk_exec) {
        cudaGraphExecDestroy(c->chunk_exec);
        c->chunk_exec = nullptr;
    }
    if (c->nbr_chunk_exec) {
        cudaGraphExecDestroy(c->nbr_chunk_exec);
        c->nbr_chunk_exec = nullptr;
    }
    if (c->ils_exec) {
        cudaGraphExecDestroy(c->ils_exec);
        c->ils_exec = nullptr;
    }
    if (c->d_tiles) {
        cudaFree(c->d_tiles);
        c->d_tiles = nullptr;
    }
    if (c->d_work) {
        cudaFree(c->d_work);
        c->d_work = nullptr;
    }
    if (c->variant == LOGO_SWEEP_BOXED && !c->d_nbr) {
        // near neighbours of every city, once per context: the boxed sweep's
        // seed pass evaluates their pairs first (host grid search)
        std::vector<logo_xy> h(c->n);
        CK(c, cudaMemcpy(h.data(), c->d_xy, sizeof(logo_xy) * c->n, cudaMemcpyDeviceToHost));
        std::vector<uint32_t> nb((size_t)c->n * kSeedNeighbours);
        knn_grid(h.data(), c->n, kSeedNeighbours, nb.data());
        CK(c, cudaMalloc(&c->d_pos, sizeof(uint32_t) * c->n));
        // positions are written by every kernel that moves the tour; until a
        // route is uploaded they only need to be in range
        CK(c, cudaMemset(c->d_pos, 0, sizeof(uint32_t) * c->n));
        CK(c, cudaMalloc(&c->d_nbr, sizeof(uint32_t) * nb.size()));
        CK(c, cudaMemcpy(c->d_nbr, nb.data(), sizeof(uint32_t) * nb.size(),
                         cudaMemcpyHostToDevice));
    }
    std::vector<uint2> tiles = make_tiles(c->n, c->R, c->NW, c->cb);
    c->ntiles = (uint32_t)tiles.size();
    if (c->ntiles) {
        CK(c, cudaMalloc(&c->d_work, sizeof(uint4) * tiles.size()));
        CK(c, cudaMalloc(&c->d_tiles, sizeof(uint2) * tiles.size()));
        CK(c, cudaMemcpy(c->d_tiles, tiles.data(), sizeof(uint2) * tiles.size(),
                         cudaMemcpyHostToDevice));
    }
    // the sweep's shared-memory opt-in must be set outside stream capture
    CK(c, launch_sweep_prepare(sweep_args(c)));
    c->chunk_steps = pick_graph_steps(c->n);
    cudaGraph_t g = nullptr;
    CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const SweepLaunch L = sweep_args(c);
    const TourBufs T = bufs(c);
    cudaError_t e = cudaSuccess;
    for (uint32_t s = 0; s < c->chunk_steps && e == cudaSuccess; ++s) {
        e = launch_sweep(L, c->stream);
        if (e == cudaSuccess) e = launch_apply_move(T, c->stream);
    }
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(c, LOGO_ERR_CUDA,
                    std::string("graph capture: ") +
                        cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&c->chunk_exec, g, 0);
    cudaGraphDestroy(g);
    CK(c, e);
    if (c->search != LOGO_SEARCH_EXHAUSTIVE) {
        g = nullptr;
        CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const NbrLaunch N = nbr_args(c);
        e = cudaSuccess;
        for (uint32_t s = 0; s < c->nbr_chunk_steps && e == cudaSuccess; ++s) {
            e = launch_nbr_sweep(N, c->stream);
            if (e == cudaSuccess) e = launch_nbr_apply(c, T, c->stream);
        }
        e2 = cudaStreamEndCapture(c->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return fail(c, LOGO_ERR_CUDA,
                        std::string("graph capture: ") +
                            cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        e = cudaGraphInstantiate(&c->nbr_chunk_exec, g, 0);
        cudaGraphDestroy(g);
        CK(c, e);
    }
    return LOGO_OK;
}

// Neighbour lists and exact positions for LOGO_SEARCH_NEIGHBOUR (host grid
// search, once per list length); graphs are rebuilt by the caller.
logo_status prepare_search(logo_ctx* c) {
    c->nbr_coop_grid =
        coop_nbr_grid(c->n, c->search == LOGO_SEARCH_NEIGHBOUR_OROPT, c->device);
    if (c->nbr_coop_grid > 0 && !c->d_coop)
        CK(c, cudaMalloc(&c->d_coop, sizeof(CoopSync)));
    if (!c->d_pos) {
        CK(c, cudaMalloc(&c->d_pos, sizeof(uint32_t) * c->n));
        CK(c, cudaMemset(c->d_pos, 0, sizeof(uint32_t) * c->n));
    }
    if (c->have_route)  // positions were not kept while nothing needed them
        CK(c, launch_fill_pos(nbr_args(c), c->stream));
    if (c->nbr_list_k != c->search_k) {
        std::vector<logo_xy> h(c->n);
        CK(c, cudaMemcpy(h.data(), c->d_xy, sizeof(logo_xy) * c->n, cudaMemcpyDeviceToHost));
        std::vector<uint32_t> nb((size_t)c->n * c->search_k);
        knn_grid(h.data(), c->n, c->search_k, nb.data());
        if (c->d_nbr_search) cudaFree(c->d_nbr_search);
        c->d_nbr_search = nullptr;
        c->nbr_list_k = 0;
        CK(c, cudaMalloc(&c->d_nbr_search, sizeof(uint32_t) * nb.size()));
        CK(c, cudaMemcpy(c->d_nbr_search, nb.data(), sizeof(uint32_t) * nb.size(),
                         cudaMemcpyHostToDevice));
        c->nbr_list_k = c->search_k;
    }
    CK(c, cudaStreamSynchronize(c->stream));
    return LOGO_OK;
}

// ---- device-run ILS graph ---------------------------------------------------
// One graph runs a whole ILS call (ILSGlobalSolverSequential::optimize,
// src/solvers/ILSGlobalSolverSequential.cpp:60-100, with a kick count):
//
//   descent_cond(first) ; WHILE(d) { chunk_steps x (sweep, apply) ; descent_cond }
//   length ; accept ; kick_cond(first)
//   WHILE(k) { kick ; descent_cond(first) ; WHILE(d2) { ... } ; length ; accept ; kick_cond }
//
// so the host launches it once and synchronises once per call.  Every loop
// is bounded on the device (descent_cond_kernel / kick_cond_kernel).

// Adds a WHILE node on handle h at the capture position of stream s and
// captures its body, built by body(bs), on stream bs.
template <typename F>
cudaError_t capture_while(cudaStream_t s, cudaGraphConditionalHandle h, cudaStream_t bs,
                          F body) {
    cudaStreamCaptureStatus cst;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, nullptr, &nd);
    if (e != cudaSuccess) return e;
    if (cst != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureInvalidated;
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &p);
    if (e != cudaSuccess) return e;
    e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                            cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(bs, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const cudaError_t eb = body(bs);
    cudaGraph_t out = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(bs, &out);
    return eb != cudaSuccess ? eb : ee;
}

// The graph currently captured on stream s (for handle creation).
cudaError_t capturing_graph(cudaStream_t s, cudaGraph_t* g) {
    cudaStreamCaptureStatus cst;
    return cudaStreamGetCaptureInfo(s, &cst, nullptr, g, nullptr, nullptr, nullptr);
}

// descent_cond(first) + WHILE(h) { steps x (sweep, apply) + descent_cond }
// at the capture position of s (graph g holds the WHILE node); bs captures
// the body.  nbr: neighbour sweeps instead of full ones.
cudaError_t capture_sweep_loop(const logo_ctx* c, cudaStream_t s, cudaGraph_t g,
                               cudaStream_t bs, bool nbr) {
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
    if (e != cudaSuccess) return e;
    e = launch_descent_cond(c->d_st, h, true, s);
    if (e != cudaSuccess) return e;
    const SweepLaunch L = sweep_args(c);
    const NbrLaunch N = nbr_args(c);
    const TourBufs T = bufs(c);
    const uint32_t steps = nbr ? c->nbr_chunk_steps : c->chunk_steps;
    DevState* st = c->d_st;
    return capture_while(s, h, bs, [&](cudaStream_t b) {
        cudaError_t eb = cudaSuccess;
        for (uint32_t k = 0; k < steps && eb == cudaSuccess; ++k) {
            eb = nbr ? launch_nbr_sweep(N, b) : launch_sweep(L, b);
            if (eb == cudaSuccess) eb = nbr ? launch_nbr_apply(c, T, b) : launch_apply_move(T, b);
        }
        if (eb == cudaSuccess) eb = launch_descent_cond(st, h, false, b);
        return eb;
    });
}

// One descent at the capture position of s: the full-sweep loop, or with
// LOGO_SEARCH_NEIGHBOUR the neighbour loop, a resume and the full loop.
cudaError_t capture_descent_loop(const logo_ctx* c, cudaStream_t s, cudaGraph_t g,
                                 cudaStream_t bs) {
    if (c->search == LOGO_SEARCH_EXHAUSTIVE) return capture_sweep_loop(c, s, g, bs, false);
    // the neighbour phase: one cooperative kernel node where available
    cudaError_t e = c->nbr_coop_grid > 0 && c->descent_mode != LOGO_DESCENT_GRAPH
                        ? launch_coop_nbr(nbr_args(c), c->d_coop, c->nbr_coop_grid, s)
                        : capture_sweep_loop(c, s, g, bs, true);
    if (e == cudaSuccess) e = launch_resume_descent(bufs(c), s);
    if (e == cudaSuccess) e = capture_sweep_loop(c, s, g, bs, false);
    return e;
}

logo_status build_ils_graph(logo_ctx* c) {
    if (c->ils_exec) return LOGO_OK;
    cudaStream_t s2 = nullptr, s3 = nullptr;
    CK(c, cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
    if (cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(s2);
        return fail(c, LOGO_ERR_CUDA, "stream creation failed");
    }
    const TourBufs T = bufs(c);
    DevState* st = c->d_st;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    cudaGraph_t top = nullptr;
    if (e == cudaSuccess) e = capturing_graph(c->stream, &top);
    if (e == cudaSuccess) e = capture_descent_loop(c, c->stream, top, s2);
    if (e == cudaSuccess) e = launch_tour_length(T, c->stream);
    if (e == cudaSuccess) e = launch_accept(T, c->stream);
    cudaGraphConditionalHandle hk;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hk, top, 0, 0);
    if (e == cudaSuccess) e = launch_kick_cond(st, hk, true, c->stream);
    if (e == cudaSuccess)
        e = capture_while(c->stream, hk, s2, [&](cudaStream_t b) {
            cudaError_t eb = launch_kick_dev(T, b);
            cudaGraph_t body = nullptr;
            if (eb == cudaSuccess) eb = capturing_graph(b, &body);
            if (eb == cudaSuccess) eb = capture_descent_loop(c, b, body, s3);
            if (eb == cudaSuccess) eb = launch_tour_length(T, b);
            if (eb == cudaSuccess) eb = launch_accept(T, b);
            if (eb == cudaSuccess) eb = launch_kick_cond(st, hk, false, b);
            return eb;
        });
    const cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    cudaStreamDestroy(s2);
    cudaStreamDestroy(s3);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return fail(c, LOGO_ERR_CUDA,
                    std::string("ILS graph capture: ") +
                        cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&c->ils_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->ils_exec = nullptr;
        return fail(c, LOGO_ERR_CUDA, std::string("ILS graph instantiation: ") +
                                          cudaGetErrorString(e));
    }
    return LOGO_OK;
}

// Route transfer: the device reads and writes the caller's buffer in place
// when it can reach pageable host memory (cudaDevAttrPageableMemoryAccess,
// e.g. over a coherent CPU-GPU link; LOGO_ROUTE_IO_AUTO), else the buffer
// is copied with cudaMemcpyAsync (LOGO_ROUTE_IO_COPY).
bool route_direct(const logo_ctx* c) {
    return c->route_io == LOGO_ROUTE_IO_DIRECT ||
           (c->route_io == LOGO_ROUTE_IO_AUTO && c->pageable_ok);
}

// Uploads a route and builds the ordered tour in one launch.  Whether the
// route is a permutation of 0..n-1 is checked on the device by the same
// launch (a host check cost about 80 us per call at n = 100k, a tenth of a
// sweep); read_state reports a bad route as LOGO_ERR_INVALID_ARG, and a
// descent on it converges before any sweep.  With reset_moves != 0 the
// launch also prepares a descent of at most reset_moves moves.
// Copy mode copies straight from the caller's buffer: measured on GB300
// (n = 100k, 400 KB) 11 us each way, against 19 us (in) and 23 us (out)
// through a pinned staging buffer and a host memcpy.
logo_status upload_route(logo_ctx* c, const uint32_t* route,
                         unsigned long long reset_moves = 0) {
    if (!route) return fail(c, LOGO_ERR_INVALID_ARG, "route is NULL");
    const uint32_t* src = route;
    if (!route_direct(c)) {
        CK(c, cudaMemcpyAsync(c->d_route[0], route, sizeof(uint32_t) * c->n,
                              cudaMemcpyHostToDevice, c->stream));
        src = c->d_route[0];
    }
    if (++c->load_epoch == 0xFFFFFFFFu) {  // every value seen holds is stale again
        CK(c, cudaMemsetAsync(c->d_seen, 0, sizeof(uint32_t) * c->n, c->stream));
        c->load_epoch = 1;
    }
    CK(c, launch_load_route(bufs(c), src, c->load_epoch, reset_moves, c->stream));
    c->have_route = true;
    return LOGO_OK;
}

logo_status read_state(logo_ctx* c) {
    CK(c, cudaMemcpyAsync(c->h_st, c->d_st, sizeof(DevState), cudaMemcpyDeviceToHost,
                          c->stream));
    ++c->host_waits;
    CK(c, cudaStreamSynchronize(c->stream));
    if (c->h_st->bad_route) {
        c->have_route = false;
        return fail(c, LOGO_ERR_INVALID_ARG, "route is not a permutation of 0..n-1");
    }
    return LOGO_OK;
}

// A device-side wait that gave up (kErrTimeout) may have left a bulk copy
// in flight into shared memory of a CTA that has already exited, or CTAs of
// a cooperative grid still running; nothing later on this context can rely
// on its buffers, so the context refuses every further call except destroy.
logo_status poisoned_error(logo_ctx* c) {
    return fail(c, LOGO_ERR_DEVICE_FAULT,
                "context unusable: a device-side wait timed out earlier; destroy it and "
                "create a new one");
}

logo_status status_to_error(logo_ctx* c, unsigned int st) {
    if (st & kErrTimeout) {
        c->poisoned = true;
        return fail(c, LOGO_ERR_TIMEOUT,
                    "a device-side wait exceeded its time budget; the context is unusable "
                    "from now on (destroy it)");
    }
    if (st & kErrBadKey)
        return fail(c, LOGO_ERR_DEVICE_FAULT, "sweep produced an out-of-range move");
    if (st & kErrMoveLimit)
        return fail(c, LOGO_ERR_MOVE_LIMIT, "descent reached max_moves");
    if (st) return fail(c, LOGO_ERR_DEVICE_FAULT, "device status " + std::to_string(st));
    return LOGO_OK;
}

// Descent on the resident tour.  Replays the chunk graph until the device
// reports convergence (or the move limit).
logo_status graph_descent(logo_ctx* c, uint64_t max_moves, bool partial_ok, uint64_t moves0,
                          uint64_t before, uint32_t* route_out, bool* route_stored,
                          bool nbr = false);
logo_status enqueue_route_out(logo_ctx* c, uint32_t* route, bool best);

// Cooperative descents of this library never overlap on one device: each
// grid is sized to be resident on its own, and two whose CTAs were only
// partly resident would wait on each other's SMs until their barriers gave
// up.  The lock is held from the launch to its completion.
std::mutex& coop_lock(int device) {
    static std::mutex locks[64];
    return locks[(unsigned)device % 64];
}

bool use_coop(const logo_ctx* c) {
    return c->coop_grid > 0 && c->descent_mode != LOGO_DESCENT_GRAPH &&
           c->search == LOGO_SEARCH_EXHAUSTIVE;
}

// reset_enqueued: the reset was folded into the route load just before.
// route_out (direct route mode only): the caller's buffer, written on the
// device before the final state read when the descent is known to end there
// (one wait instead of two); *route_stored says whether it was.
logo_status run_descent(logo_ctx* c, uint64_t max_moves, uint64_t* moves_out,
                        uint64_t* sweeps_out, bool reset = true, bool reset_enqueued = false,
                        uint32_t* route_out = nullptr, bool* route_stored = nullptr) {
    if (max_moves == 0) max_moves = ~0ull >> 1;
    if (route_stored) *route_stored = false;
    if (reset && !reset_enqueued)  // also clears the status word
        CK(c, launch_reset_descent(bufs(c), max_moves, c->stream));
    else if (!reset)
        CK(c, cudaMemsetAsync(&c->d_st->status, 0, sizeof(unsigned int), c->stream));
    // a fresh descent starts from zero moves and records its sweep count on
    // the device; a continued one needs the counters first
    uint64_t moves0 = 0, sweeps0 = 0;
    if (!reset) {
        logo_status s0 = read_state(c);
        if (s0 != LOGO_OK) return s0;
        moves0 = c->h_st->moves;
        sweeps0 = c->h_st->sweeps;
    }
    if (use_coop(c)) {
        // one cooperative launch runs the whole descent
        CK(c, cudaMemsetAsync(c->d_coop, 0xFF, sizeof(CoopSync), c->stream));
        CK(c, cudaMemsetAsync(c->d_coop, 0, 2 * sizeof(unsigned int), c->stream));
        CoopArgs A;
        A.Q0 = c->d_Q[0];
        A.Q1 = c->d_Q[1];
        A.R0 = c->d_route[0];
        A.R1 = c->d_route[1];
        A.n = c->n;
        A.margin = c->margin;
        A.st = c->d_st;
        A.cs = c->d_coop;
        logo_status s;
        {
            std::lock_guard<std::mutex> lk(coop_lock(c->device));
            CK(c, launch_coop_descent(A, c->coop_grid, c->stream));
            if (route_out) {  // the launch runs the whole descent
                s = enqueue_route_out(c, route_out, false);
                if (s != LOGO_OK) return s;
                if (route_stored) *route_stored = true;
            }
            s = read_state(c);
        }
        if (s != LOGO_OK) return s;
        if (!c->h_st->converged && !c->h_st->status)
            return fail(c, LOGO_ERR_DEVICE_FAULT, "cooperative descent did not finish");
    } else if (c->search != LOGO_SEARCH_EXHAUSTIVE) {
        // neighbour sweeps until no candidate improves (one cooperative
        // launch where available), then full sweeps
        logo_status s;
        if (c->nbr_coop_grid > 0 && c->descent_mode != LOGO_DESCENT_GRAPH) {
            CK(c, cudaMemsetAsync(c->d_coop, 0xFF, sizeof(CoopSync), c->stream));
            CK(c, cudaMemsetAsync(c->d_coop, 0, 2 * sizeof(unsigned int), c->stream));
            std::lock_guard<std::mutex> lk(coop_lock(c->device));
            CK(c, launch_coop_nbr(nbr_args(c), c->d_coop, c->nbr_coop_grid, c->stream));
            s = read_state(c);
        } else {
            s = graph_descent(c, max_moves, reset, moves0, moves0, nullptr, nullptr, true);
        }
        if (s != LOGO_OK) return s;
        if (!c->h_st->status && !c->h_st->bad_route) {
            CK(c, launch_resume_descent(bufs(c), c->stream));
            s = graph_descent(c, max_moves, reset, moves0, c->h_st->moves, route_out,
                              route_stored);
            if (s != LOGO_OK) return s;
        }
    } else {
        logo_status s = graph_descent(c, max_moves, reset, moves0, moves0, route_out,
                                      route_stored);
        if (s != LOGO_OK) return s;
    }
    if (moves_out) *moves_out = c->h_st->moves - moves0;
    if (sweeps_out)
        *sweeps_out = c->h_st->sweeps - (reset ? c->h_st->sweeps_at_reset : sweeps0);
    const unsigned int st = c->h_st->status & ~kErrMoveLimit;
    if (st) return status_to_error(c, st);
    return LOGO_OK;
}

// Replays the chunk graph (or single steps when fewer moves are allowed than
// a chunk holds) until the device flags convergence.
logo_status graph_descent(logo_ctx* c, uint64_t max_moves, bool partial_ok, uint64_t moves0,
                          uint64_t before, uint32_t* route_out, bool* route_stored, bool nbr) {
    const uint32_t chunk = nbr ? c->nbr_chunk_steps : c->chunk_steps;
    for (;;) {
        const uint64_t left = max_moves - (before - moves0);
        bool stored = false;
        if (partial_ok && left < chunk) {
            // fewer moves allowed than a chunk holds: launch just those steps,
            // after which the descent (or its neighbour phase) has converged
            // or met its move limit
            const SweepLaunch L = sweep_args(c);
            const NbrLaunch N = nbr_args(c);
            const TourBufs T = bufs(c);
            for (uint64_t k = 0; k < left; ++k) {
                CK(c, nbr ? launch_nbr_sweep(N, c->stream) : launch_sweep(L, c->stream));
                // the last full-sweep step also hands the tour back (direct mode)
                uint32_t* out = !nbr && route_out && k + 1 == left ? route_out : nullptr;
                CK(c, nbr ? launch_nbr_apply(c, T, c->stream)
                          : launch_apply_move(T, c->stream, out));
                stored = stored || out != nullptr;
            }
            if (route_out && !stored) {
                logo_status s = enqueue_route_out(c, route_out, false);
                if (s != LOGO_OK) return s;
                stored = true;
            }
        } else {
            CK(c, cudaGraphLaunch(nbr ? c->nbr_chunk_exec : c->chunk_exec, c->stream));
        }
        logo_status s = read_state(c);
        if (s != LOGO_OK) return s;
        if (c->h_st->converged || c->h_st->status) {
            if (route_stored) *route_stored = stored;
            break;
        }
        // every replay applies at least one move or converges
        if (c->h_st->moves == before)
            return fail(c, LOGO_ERR_DEVICE_FAULT, "descent made no progress");
        before = c->h_st->moves;
    }
    return LOGO_OK;
}

// Enqueues the transfer of the current (or best) tour into the caller's
// buffer; download_route also waits for it.  Copy mode reads the current
// buffer index from the last read_state.
logo_status enqueue_route_out(logo_ctx* c, uint32_t* route, bool best) {
    if (route_direct(c)) {
        CK(c, launch_store_route(bufs(c), route, best, c->stream));
        return LOGO_OK;
    }
    const uint32_t* src = best ? c->d_route_best : c->d_route[c->h_st->cur & 1];
    CK(c, cudaMemcpyAsync(route, src, sizeof(uint32_t) * c->n, cudaMemcpyDeviceToHost,
                          c->stream));
    return LOGO_OK;
}

logo_status download_route(logo_ctx* c, uint32_t* route, bool best) {
    logo_status s = enqueue_route_out(c, route, best);
    if (s != LOGO_OK) return s;
    ++c->host_waits;
    CK(c, cudaStreamSynchronize(c->stream));
    return LOGO_OK;
}

logo_status length_now(logo_ctx* c, uint64_t* len) {
    CK(c, launch_tour_length(bufs(c), c->stream));
    logo_status s = read_state(c);
    if (s != LOGO_OK) return s;
    *len = c->h_st->length;
    return LOGO_OK;
}

void destroy(logo_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->chunk_exec) cudaGraphExecDestroy(c->chunk_exec);
    if (c->ils_exec) cudaGraphExecDestroy(c->ils_exec);
    cudaFree(c->d_xy);
    cudaFree(c->d_Q[0]);
    cudaFree(c->d_Q[1]);
    cudaFree(c->d_route[0]);
    cudaFree(c->d_route[1]);
    cudaFree(c->d_Qbest);
    cudaFree(c->d_route_best);
    cudaFree(c->d_st);
    cudaFree(c->d_tiles);
    cudaFree(c->d_seen);
    cudaFree(c->d_wbox);
    cudaFree(c->d_wmax);
    cudaFree(c->d_rbox);
    cudaFree(c->d_rmax);
    cudaFree(c->d_work);
    cudaFree(c->d_workctl);
    cudaFree(c->d_pos);
    cudaFree(c->d_nbr);
    cudaFree(c->d_nbr_search);
    cudaFree(c->d_start);
    if (c->nbr_chunk_exec) cudaGraphExecDestroy(c->nbr_chunk_exec);
    cudaFree(c->d_coop);
    if (c->h_st) cudaFreeHost(c->h_st);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

// Device time of a call (CUDA events on the context's stream); a timer made
// with on = false records nothing and stop() returns 0 without waiting.
struct Timer {
    logo_ctx* c;
    bool on;
    explicit Timer(logo_ctx* cc, bool enabled = true) : c(cc), on(enabled) {
        if (on) cudaEventRecord(c->ev0, c->stream);
    }
    double stop() {
        if (!on) return 0.0;
        cudaEventRecord(c->ev1, c->stream);
        ++c->host_waits;
        cudaEventSynchronize(c->ev1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        return ms;
    }
};

}  // namespace

namespace logo {

// |exact delta - approximate delta| <= filter_margin(diag) for every pair of
// an instance whose bounding-box diagonal is diag.  Per distance d <= diag:
// the nint is within 0.5 + 2^-23 (d + 1) of sqrt(s); the contracted sum of
// squares is within 2^-23 s of the exact binary32 one; the MUFU square root
// is within rel_err * d of the true root (rel_err = 2^-20, at least 8x the
// error measured over all binary32 inputs by tests/test_gpu_sqrt_bound.py).
// Two distances enter a delta, and the filter's own float arithmetic
// (three roundings on magnitudes <= 4 diag) adds 3 * 2^-24 * 4 diag.  One
// unit of slack covers the strict comparison.
float filter_margin(double diag) {
    const double rel = std::ldexp(1.0, -20);
    const double u = std::ldexp(1.0, -24);
    const double m = 1.0 + 2.0 * diag * (3.0 * u + rel) + 2.0 * std::ldexp(1.0, -23) +
                     3.0 * u * 4.0 * diag + 1.0;
    return (float)m;
}

}  // namespace logo

extern "C" {

const char* logo_version(void) { return kVersion; }

const char* logo_last_error(const logo_ctx* ctx) {
    if (ctx) return ctx->err.c_str();
    return g_create_err.c_str();
}

logo_status logo_ctx_create(int device, const logo_xy* coords, uint32_t n, logo_ctx** out) {
    if (!out) return fail(nullptr, LOGO_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!coords) return fail(nullptr, LOGO_ERR_INVALID_ARG, "coords is NULL");
    if (n < 3 || n > LOGO_MAX_CITIES)
        return fail(nullptr, LOGO_ERR_INVALID_ARG,
                    "n must be in [3, " + std::to_string(LOGO_MAX_CITIES) + "]");
    double x0 = coords[0].x, x1 = coords[0].x, y0 = coords[0].y, y1 = coords[0].y;
    for (uint32_t k = 0; k < n; ++k) {
        const double x = coords[k].x, y = coords[k].y;
        if (!std::isfinite(x) || !std::isfinite(y))
            return fail(nullptr, LOGO_ERR_INVALID_ARG,
                        "coordinate " + std::to_string(k) + " is not finite");
        x0 = std::min(x0, x); x1 = std::max(x1, x);
        y0 = std::min(y0, y); y1 = std::max(y1, y);
    }
    const double diag = std::sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0));
    if (!(diag < LOGO_MAX_DIAGONAL))
        return fail(nullptr, LOGO_ERR_INVALID_ARG,
                    "coordinate bounding-box diagonal exceeds LOGO_MAX_DIAGONAL");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, LOGO_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev)
        return fail(nullptr, LOGO_ERR_INVALID_ARG, "device index out of range");
    if (cudaSetDevice(device) != cudaSuccess)
        return fail(nullptr, LOGO_ERR_CUDA, "cudaSetDevice failed");

    logo_ctx* c = new logo_ctx();
    c->device = device;
    c->n = n;
    c->diag = diag;
    c->margin = filter_margin(diag);
    default_shape(n, c->R, c->NW, c->cb, c->variant);
    logo_status s = LOGO_OK;
    auto bail = [&](logo_status st) {
        g_create_err = c->err;
        destroy(c);
        return st;
    };
#define CKC(call)                                                             \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) {                                              \
            c->err = std::string(#call) + ": " + cudaGetErrorString(e_);      \
            return bail(e_ == cudaErrorMemoryAllocation ? LOGO_ERR_OOM         \
                                                        : LOGO_ERR_CUDA);     \
        }                                                                     \
    } while (0)
    CKC(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CKC(cudaEventCreate(&c->ev0));
    CKC(cudaEventCreate(&c->ev1));
    CKC(cudaMalloc(&c->d_xy, sizeof(float2) * n));
    for (int b = 0; b < 2; ++b) {
        CKC(cudaMalloc(&c->d_Q[b], sizeof(OrderedCity) * n));
        CKC(cudaMalloc(&c->d_route[b], sizeof(uint32_t) * n));
    }
    CKC(cudaMalloc(&c->d_Qbest, sizeof(OrderedCity) * n));
    CKC(cudaMalloc(&c->d_route_best, sizeof(uint32_t) * n));
    CKC(cudaMalloc(&c->d_st, sizeof(DevState)));
    CKC(cudaMallocHost(&c->h_st, sizeof(DevState)));
    CKC(cudaMalloc(&c->d_seen, sizeof(uint32_t) * n));
    CKC(cudaMemset(c->d_seen, 0, sizeof(uint32_t) * n));
    {
        int pageable = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) !=
            cudaSuccess)
            pageable = 0;
        c->pageable_ok = pageable != 0;
    }
    CKC(cudaMalloc(&c->d_wbox, sizeof(float4) * sweep_windows(n)));
    CKC(cudaMalloc(&c->d_wmax, sizeof(float) * sweep_windows(n)));
    CKC(cudaMalloc(&c->d_rbox, sizeof(float4) * sweep_row_windows(n)));
    CKC(cudaMalloc(&c->d_rmax, sizeof(float) * sweep_row_windows(n)));
    CKC(cudaMalloc(&c->d_workctl, 3 * sizeof(uint32_t)));
    c->coop_grid = coop_grid(n, device);
    c->coop_ils_grid = c->coop_grid > 0 ? coop_ils_grid(n, device) : 0;
    if (c->coop_grid > 0) CKC(cudaMalloc(&c->d_coop, sizeof(CoopSync)));
    std::memset(c->h_st, 0, sizeof(DevState));
    c->h_st->best_key = kNoMove;
    c->h_st->converged = 1;
    CKC(cudaMemcpy(c->d_st, c->h_st, sizeof(DevState), cudaMemcpyHostToDevice));
    CKC(cudaMemcpy(c->d_xy, coords, sizeof(float2) * n, cudaMemcpyHostToDevice));
#undef CKC
    s = rebuild(c);
    if (s != LOGO_OK) return bail(s);
    *out = c;
    return LOGO_OK;
}

logo_status logo_ctx_destroy(logo_ctx* ctx) {
    destroy(ctx);
    return LOGO_OK;
}

logo_status logo_ctx_get_info(const logo_ctx* c, logo_ctx_info* info) {
    if (!c || !info) return LOGO_ERR_INVALID_ARG;
    info->n = c->n;
    info->device = c->device;
    info->rows_per_thread = c->R;
    info->warps_per_cta = c->NW;
    info->tile_cols = c->cb;
    info->tiles = c->ntiles;
    info->filter_margin = c->margin;
    info->graph_steps = c->chunk_steps;
    info->variant = c->variant;
    info->descent_mode = use_coop(c) ? LOGO_DESCENT_COOPERATIVE : LOGO_DESCENT_GRAPH;
    info->cooperative_ctas = c->coop_grid;
    info->host_waits = c->host_waits;
    info->route_io = route_direct(c) ? LOGO_ROUTE_IO_DIRECT : LOGO_ROUTE_IO_COPY;
    info->search = c->search;
    info->search_neighbours = c->search_k;
    info->pad0 = 0;
    return LOGO_OK;
}

logo_status logo_start_tour(logo_ctx* c, int kind, uint32_t* route) {
    if (!c || !route) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (kind != LOGO_START_NN && kind != LOGO_START_MF)
        return fail(c, LOGO_ERR_INVALID_ARG, "unknown start-tour kind");
    if (c->n > LOGO_BATCH_MAX_N)
        return fail(c, LOGO_ERR_INVALID_ARG,
                    "device start tours hold the instance in one CTA (up to " +
                        std::to_string(LOGO_BATCH_MAX_N) +
                        " cities); larger tours: logo_nn_tour / logo_mf_tour");
    CK(c, cudaSetDevice(c->device));
    if (!c->d_start) CK(c, cudaMalloc(&c->d_start, sizeof(uint32_t) * c->n));
    CK(c, launch_start_tour(c->d_xy, c->n, kind == LOGO_START_NN ? kStartNN : kStartMF,
                            c->d_start, c->stream));
    CK(c, cudaMemcpyAsync(route, c->d_start, sizeof(uint32_t) * c->n, cudaMemcpyDeviceToHost,
                          c->stream));
    ++c->host_waits;
    CK(c, cudaStreamSynchronize(c->stream));
    return LOGO_OK;
}

logo_status logo_ctx_set_search(logo_ctx* c, int mode, uint32_t neighbours) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (mode != LOGO_SEARCH_EXHAUSTIVE && mode != LOGO_SEARCH_NEIGHBOUR &&
        mode != LOGO_SEARCH_NEIGHBOUR_OROPT)
        return fail(c, LOGO_ERR_INVALID_ARG, "unknown search mode");
    if (neighbours == 0) neighbours = kSearchNeighbours;
    if (neighbours > kSearchNeighboursMax)
        return fail(c, LOGO_ERR_INVALID_ARG,
                    "neighbour lists hold at most " + std::to_string(kSearchNeighboursMax) +
                        " cities");
    CK(c, cudaSetDevice(c->device));
    CK(c, cudaStreamSynchronize(c->stream));
    c->search = mode;
    c->search_k = neighbours;
    if (mode != LOGO_SEARCH_EXHAUSTIVE) {
        logo_status s = prepare_search(c);
        if (s != LOGO_OK) return s;
    }
    return rebuild(c);
}

logo_status logo_ctx_set_route_io(logo_ctx* c, int mode) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (mode != LOGO_ROUTE_IO_AUTO && mode != LOGO_ROUTE_IO_COPY &&
        mode != LOGO_ROUTE_IO_DIRECT)
        return fail(c, LOGO_ERR_INVALID_ARG, "unknown route transfer mode");
    if (mode == LOGO_ROUTE_IO_DIRECT && !c->pageable_ok)
        return fail(c, LOGO_ERR_INVALID_ARG,
                    "direct route transfer unavailable: the device cannot access pageable "
                    "host memory");
    c->route_io = mode;
    return LOGO_OK;
}

logo_status logo_ctx_set_descent_mode(logo_ctx* c, int mode) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (mode != LOGO_DESCENT_AUTO && mode != LOGO_DESCENT_GRAPH &&
        mode != LOGO_DESCENT_COOPERATIVE)
        return fail(c, LOGO_ERR_INVALID_ARG, "unknown descent mode");
    if (mode == LOGO_DESCENT_COOPERATIVE && c->coop_grid <= 0)
        return fail(c, LOGO_ERR_INVALID_ARG,
                    "cooperative descent unavailable (n above 6,144 or device without it)");
    c->descent_mode = mode;
    return LOGO_OK;
}

logo_status logo_ctx_set_shape(logo_ctx* c, int R, int NW, uint32_t cb) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!sweep_shape_supported(R, NW, c->variant) || cb < 16 || cb > 4096 ||
        !sweep_cols_supported(c->variant, cb))
        return fail(c, LOGO_ERR_INVALID_ARG, "unsupported sweep shape");
    CK(c, cudaSetDevice(c->device));
    CK(c, cudaStreamSynchronize(c->stream));
    c->R = R;
    c->NW = NW;
    c->cb = cb;
    return rebuild(c);
}

logo_status logo_ctx_set_kernel(logo_ctx* c, int variant, int R, int NW, uint32_t cb) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (variant < LOGO_SWEEP_MUFU || variant > LOGO_SWEEP_BOXED ||
        (variant > LOGO_SWEEP_MUFU && variant < LOGO_SWEEP_FUSED))
        return fail(c, LOGO_ERR_INVALID_ARG, "unknown or retired sweep variant");
    if (!sweep_shape_supported(R, NW, variant) || cb < 16 || cb > 4096 ||
        !sweep_cols_supported(variant, cb))
        return fail(c, LOGO_ERR_INVALID_ARG, "unsupported sweep shape for this variant");
    CK(c, cudaSetDevice(c->device));
    CK(c, cudaStreamSynchronize(c->stream));
    c->variant = variant;
    c->R = R;
    c->NW = NW;
    c->cb = cb;
    return rebuild(c);
}

void* logo_ctx_stream(logo_ctx* c) { return c ? (void*)c->stream : nullptr; }

logo_status logo_sync(logo_ctx* c) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    CK(c, cudaStreamSynchronize(c->stream));
    return LOGO_OK;
}

logo_status logo_begin_descent(logo_ctx* c, uint64_t max_moves) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!c->have_route) return fail(c, LOGO_ERR_INVALID_ARG, "no resident route");
    CK(c, cudaSetDevice(c->device));
    if (max_moves == 0) max_moves = ~0ull >> 1;
    CK(c, launch_reset_descent(bufs(c), max_moves, c->stream));  // clears status too
    return LOGO_OK;
}

logo_status logo_enqueue_sweep(logo_ctx* c) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!c->have_route) return fail(c, LOGO_ERR_INVALID_ARG, "no resident route");
    CK(c, cudaSetDevice(c->device));
    CK(c, launch_sweep(sweep_args(c), c->stream));
    return LOGO_OK;
}

logo_status logo_enqueue_apply(logo_ctx* c) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!c->have_route) return fail(c, LOGO_ERR_INVALID_ARG, "no resident route");
    CK(c, cudaSetDevice(c->device));
    CK(c, launch_apply_move(bufs(c), c->stream));
    return LOGO_OK;
}

logo_status logo_get_progress(logo_ctx* c, uint64_t* moves, int* converged) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    CK(c, cudaSetDevice(c->device));
    logo_status s = read_state(c);
    if (s != LOGO_OK) return s;
    if (moves) *moves = c->h_st->moves;
    if (converged) *converged = c->h_st->converged ? 1 : 0;
    const unsigned int st = c->h_st->status & ~kErrMoveLimit;
    if (st) return status_to_error(c, st);
    return LOGO_OK;
}

logo_status logo_diag_flag_timeout(logo_ctx* c) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    CK(c, cudaSetDevice(c->device));
    const unsigned int bit = kErrTimeout;
    CK(c, cudaMemcpyAsync(&c->d_st->status, &bit, sizeof(bit), cudaMemcpyHostToDevice,
                          c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return LOGO_OK;
}

logo_status logo_set_route(logo_ctx* c, const uint32_t* route) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    CK(c, cudaSetDevice(c->device));
    logo_status s = upload_route(c, route);
    if (s != LOGO_OK) return s;
    return read_state(c);
}

logo_status logo_get_route(logo_ctx* c, uint32_t* route) {
    if (!c || !route) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!c->have_route) return fail(c, LOGO_ERR_INVALID_ARG, "no resident route");
    CK(c, cudaSetDevice(c->device));
    logo_status s = read_state(c);
    if (s != LOGO_OK) return s;
    return download_route(c, route, false);
}

static logo_status sweep_once(logo_ctx* c, logo_move* out, bool reset_enqueued);

logo_status logo_best_move(logo_ctx* c, const uint32_t* route, logo_move* out) {
    if (!c || !out) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    CK(c, cudaSetDevice(c->device));
    logo_status s = upload_route(c, route, ~0ull >> 1);
    if (s != LOGO_OK) return s;
    return sweep_once(c, out, true);
}

logo_status logo_sweep_resident(logo_ctx* c, logo_move* out) {
    if (!c || !out) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!c->have_route) return fail(c, LOGO_ERR_INVALID_ARG, "no resident route");
    CK(c, cudaSetDevice(c->device));
    return sweep_once(c, out, false);
}

static logo_status sweep_once(logo_ctx* c, logo_move* out, bool reset_enqueued) {
    if (!reset_enqueued)
        CK(c, launch_reset_descent(bufs(c), ~0ull >> 1, c->stream));  // clears status too
    CK(c, launch_sweep(sweep_args(c), c->stream));
    logo_status s = read_state(c);
    if (s != LOGO_OK) return s;
    if (c->h_st->status) return status_to_error(c, c->h_st->status);
    const uint64_t k = c->h_st->best_key;
    if (k == kNoMove) {
        out->i = 0;
        out->j = 0;
        out->minchange = 0;
    } else {
        out->i = key_i(k);
        out->j = key_j(k);
        out->minchange = key_delta(k);
    }
    return LOGO_OK;
}

logo_status logo_descend_resident(logo_ctx* c, uint64_t max_moves, logo_stats* stats) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!c->have_route) return fail(c, LOGO_ERR_INVALID_ARG, "no resident route");
    CK(c, cudaSetDevice(c->device));
    Timer t(c);
    uint64_t moves = 0, sweeps = 0;
    logo_status s = run_descent(c, max_moves, &moves, &sweeps);
    const double ms = t.stop();
    if (s != LOGO_OK) return s;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->moves = moves;
        stats->sweeps = sweeps;
        stats->pair_evals = pair_evals_of(c, sweeps, c->h_st->nbr_sweeps);
        stats->descents = 1;
        stats->device_ms = ms;
    }
    return LOGO_OK;
}

logo_status logo_length_resident(logo_ctx* c, uint64_t* len) {
    if (!c || !len) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (!c->have_route) return fail(c, LOGO_ERR_INVALID_ARG, "no resident route");
    CK(c, cudaSetDevice(c->device));
    return length_now(c, len);
}

logo_status logo_tour_length(logo_ctx* c, const uint32_t* route, uint64_t* len) {
    if (!c || !len) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    CK(c, cudaSetDevice(c->device));
    logo_status s = upload_route(c, route);
    if (s != LOGO_OK) return s;
    return length_now(c, len);
}

static logo_status descend_impl(logo_ctx* c, uint32_t* route, uint64_t max_moves,
                                int32_t* trace, uint64_t trace_cap, logo_stats* stats) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    CK(c, cudaSetDevice(c->device));
    Timer t(c, stats != nullptr);  // no stats: no timing and no extra wait
    // without stats or a trace nothing runs between the load and the descent:
    // the load also resets the descent, and in direct route mode the result
    // is written back before the one final wait
    const bool quick = !stats && !(trace && trace_cap);
    logo_status s = upload_route(c, route, quick ? (max_moves ? max_moves : ~0ull >> 1) : 0);
    if (s != LOGO_OK) return s;
    uint64_t start_len = 0, final_len = 0, moves = 0, sweeps = 0;
    if (stats) {
        s = length_now(c, &start_len);
        if (s != LOGO_OK) return s;
    }
    int* d_log = nullptr;
    if (trace && trace_cap) {
        if (trace_cap > 0xFFFFFFFFull / 3) trace_cap = 0xFFFFFFFFull / 3;
        CK(c, cudaMalloc(&d_log, sizeof(int) * 3 * trace_cap));
        const unsigned int cap32 = (unsigned int)trace_cap;
        CK(c, cudaMemcpyAsync(&c->d_st->move_log, &d_log, sizeof(d_log),
                              cudaMemcpyHostToDevice, c->stream));
        CK(c, cudaMemcpyAsync(&c->d_st->log_cap, &cap32, sizeof(cap32),
                              cudaMemcpyHostToDevice, c->stream));
    }
    bool stored = false;
    s = run_descent(c, max_moves, &moves, &sweeps, true, quick,
                    quick && route_direct(c) ? route : nullptr, &stored);
    const uint64_t nbr_sweeps = c->h_st->nbr_sweeps;
    if (d_log) {
        int* null_log = nullptr;
        const unsigned int zero = 0;
        cudaMemcpyAsync(&c->d_st->move_log, &null_log, sizeof(null_log),
                        cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(&c->d_st->log_cap, &zero, sizeof(zero), cudaMemcpyHostToDevice,
                        c->stream);
        const uint64_t got = std::min<uint64_t>(moves, trace_cap);
        cudaError_t e = cudaMemcpyAsync(trace, d_log, sizeof(int) * 3 * got,
                                        cudaMemcpyDeviceToHost, c->stream);
        cudaStreamSynchronize(c->stream);
        cudaFree(d_log);
        if (s == LOGO_OK && e != cudaSuccess)
            return fail(c, LOGO_ERR_CUDA, "trace copy failed");
    }
    if (s != LOGO_OK) return s;
    if (stats) {
        s = length_now(c, &final_len);
        if (s != LOGO_OK) return s;
    }
    if (!stored) s = download_route(c, route, false);
    const double ms = t.stop();
    if (s != LOGO_OK) return s;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->moves = moves;
        stats->sweeps = sweeps;
        stats->pair_evals = pair_evals_of(c, sweeps, nbr_sweeps);
        stats->descents = 1;
        stats->start_length = start_len;
        stats->final_length = final_len;
        stats->device_ms = ms;
    }
    return LOGO_OK;
}

logo_status logo_descend(logo_ctx* c, uint32_t* route, uint64_t max_moves,
                         logo_stats* stats) {
    return descend_impl(c, route, max_moves, nullptr, 0, stats);
}

logo_status logo_descend_trace(logo_ctx* c, uint32_t* route, uint64_t max_moves,
                               int32_t* trace, uint64_t trace_cap, logo_stats* stats) {
    if (!trace && trace_cap) return fail(c, LOGO_ERR_INVALID_ARG, "trace is NULL");
    return descend_impl(c, route, max_moves, trace, trace_cap, stats);
}

logo_status logo_ils(logo_ctx* c, uint32_t* route, uint32_t kicks, uint64_t seed,
                     int kick_kind, logo_stats* stats) {
    if (!c) return LOGO_ERR_INVALID_ARG;
    if (c->poisoned) return poisoned_error(c);
    if (kick_kind != LOGO_KICK_SEGMENT && kick_kind != LOGO_KICK_DOUBLE_BRIDGE)
        return fail(c, LOGO_ERR_INVALID_ARG, "unknown kick kind");
    CK(c, cudaSetDevice(c->device));
    const bool coop = use_coop(c) && c->coop_ils_grid > 0;
    if (!coop) {
        logo_status sb = build_ils_graph(c);  // once per context and tile shape
        if (sb != LOGO_OK) return sb;
    }
    Timer t(c);
    logo_status s = upload_route(c, route);
    if (s != LOGO_OK) return s;
    // seed the device PRNG, clear the ILS counters, set the kick count and kind
    const unsigned long long target = kicks;
    const unsigned int kind = (unsigned int)kick_kind;
    CK(c, cudaMemcpyAsync(&c->d_st->rng, &seed, sizeof(seed), cudaMemcpyHostToDevice,
                          c->stream));
    CK(c, cudaMemcpyAsync(&c->d_st->kick_target, &target, sizeof(target),
                          cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(&c->d_st->kick_kind, &kind, sizeof(kind), cudaMemcpyHostToDevice,
                          c->stream));
    CK(c, cudaMemsetAsync(&c->d_st->total_moves, 0, sizeof(unsigned long long), c->stream));
    CK(c, cudaMemsetAsync(&c->d_st->accepted, 0, sizeof(unsigned long long), c->stream));
    CK(c, cudaMemsetAsync(&c->d_st->kicks, 0, sizeof(unsigned long long), c->stream));
    CK(c, cudaMemsetAsync(&c->d_st->sweeps, 0, sizeof(unsigned long long), c->stream));
    CK(c, launch_tour_length(bufs(c), c->stream));
    CK(c, launch_save_best(bufs(c), c->stream));  // best = start, start_length recorded
    const uint64_t kmax = 64ull * c->n * c->n + 1024;
    CK(c, launch_reset_descent(bufs(c), kmax, c->stream));
    if (coop) {
        // one cooperative launch runs every descent, length, accept and kick
        CK(c, cudaMemsetAsync(c->d_coop, 0xFF, sizeof(CoopSync), c->stream));
        CK(c, cudaMemsetAsync(c->d_coop, 0, 2 * sizeof(unsigned int), c->stream));
        CoopArgs A;
        A.Q0 = c->d_Q[0];
        A.Q1 = c->d_Q[1];
        A.R0 = c->d_route[0];
        A.R1 = c->d_route[1];
        A.n = c->n;
        A.margin = c->margin;
        A.st = c->d_st;
        A.cs = c->d_coop;
        A.xy = c->d_xy;
        A.Qbest = c->d_Qbest;
        A.route_best = c->d_route_best;
        A.kicks = kicks;
        A.kick_kind = kick_kind;
        std::lock_guard<std::mutex> lk(coop_lock(c->device));
        CK(c, launch_coop_ils(A, c->coop_ils_grid, c->stream));
        s = read_state(c);
    } else {
        // one graph: descent and kick loops are WHILE nodes on device conditions
        const bool nbr_coop = c->search != LOGO_SEARCH_EXHAUSTIVE && c->nbr_coop_grid > 0 &&
                              c->descent_mode != LOGO_DESCENT_GRAPH;
        if (nbr_coop) {  // the neighbour phases are cooperative kernel nodes
            CK(c, cudaMemsetAsync(c->d_coop, 0xFF, sizeof(CoopSync), c->stream));
            CK(c, cudaMemsetAsync(c->d_coop, 0, 2 * sizeof(unsigned int), c->stream));
            std::lock_guard<std::mutex> lk(coop_lock(c->device));
            CK(c, cudaGraphLaunch(c->ils_exec, c->stream));
            s = read_state(c);
        } else {
            CK(c, cudaGraphLaunch(c->ils_exec, c->stream));
            s = read_state(c);
        }
    }
    if (s != LOGO_OK) return s;
    const DevState fin = *c->h_st;
    const unsigned int st = fin.status & ~kErrMoveLimit;
    if (st) return status_to_error(c, st);
    if (!fin.converged || fin.kicks != kicks)
        return fail(c, LOGO_ERR_DEVICE_FAULT, "device ILS did not finish");
    s = download_route(c, route, true);
    const double ms = t.stop();
    if (s != LOGO_OK) return s;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->moves = fin.total_moves;
        stats->sweeps = fin.sweeps;
        stats->pair_evals = pair_evals_of(c, fin.sweeps, fin.nbr_sweeps);
        stats->descents = (uint64_t)kicks + 1;
        stats->kicks = fin.kicks;
        stats->accepted = fin.accepted;
        stats->start_length = fin.start_length;
        stats->final_length = fin.best_length;
        stats->device_ms = ms;
    }
    return LOGO_OK;
}

}  // extern "C"
