/*
 * logo_gpu.h -- C ABI of the GB300 (sm_103a) 2-opt local-search engine.
 *
 * Drop-in for the 2-opt hot path of the LOGO TSP solver (krocki/
 * LOGO-TSP-Solver v0.62).  The reference reaches its CUDA backend through the
 * C++ LocalSolver interface (src/solvers/localSolver.h:25-132) and calls the
 * CUDA runtime directly from CUDASolver (src/solvers/CUDASolver.cpp); this
 * header is the plain-C boundary that replaces that backend.  No torch or
 * CUDA types appear in the signatures: coordinates, routes and results are
 * host arrays owned by the caller, and every call returns a logo_status
 * (the reference prints and exit(-1)s instead, src/utils/UtilsCUDA.cpp:318-328).
 *
 * Arithmetic contract.  Distances are the reference's per-edge EUC_2D nint
 * (int)(sqrtf(dx*dx + dy*dy) + 0.5f)   (src/cuda/cuda_common.h:33-40,
 * src/headers.h:126-133) evaluated in IEEE binary32 without FMA contraction
 * and with a correctly rounded sqrt.  Moves are chosen best-improvement over
 * tour positions 1 <= i < j <= n-2 with the lowest-(i, j) tie rule of the
 * reference CPU solver (src/solvers/cpuSolver.cpp:188-230) and applied as
 * rotate-then-reverse (src/solvers/twoOptLocalSolver.cpp:41-48), so every
 * move, tour and length is bit-identical to the reference CPU path with that
 * distance.
 *
 * Limits.  3 <= n <= LOGO_MAX_CITIES; all coordinates finite; the bounding
 * box diagonal of the coordinates below LOGO_MAX_DIAGONAL (the packed argmin
 * key stores delta in 22 bits).
 *
 * Threading.  A logo_ctx belongs to one host thread at a time; it owns one
 * CUDA stream on its device.  Different contexts may be used concurrently.
 */
#ifndef LOGO_GPU_H
#define LOGO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LOGO_MAX_CITIES 2097152u   /* MAX_CITIES, src/defs.h:25 */
#define LOGO_MAX_DIAGONAL 2000000.0

typedef enum logo_status {
    LOGO_OK = 0,
    LOGO_ERR_INVALID_ARG = 1,  /* bad pointer, size, route or coordinates */
    LOGO_ERR_OOM = 2,          /* device or pinned-host allocation failed */
    LOGO_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    LOGO_ERR_TIMEOUT = 4,      /* a bounded device-side wait ran out */
    LOGO_ERR_DEVICE_FAULT = 5, /* the device status word reports an error */
    LOGO_ERR_MOVE_LIMIT = 6,   /* a descent reached its max_moves */
    LOGO_ERR_NO_DEVICE = 7,    /* no usable CUDA device */
    LOGO_ERR_BUSY = 8,         /* server queue full / slot unavailable */
    LOGO_ERR_NOT_FOUND = 9     /* unknown request id */
} logo_status;

/* city_coords, src/defs.h:173-178 */
typedef struct logo_xy {
    float x;
    float y;
} logo_xy;

/* best2_out, src/defs.h:181-187: the reported move (i, j) deletes tour edges
 * (i-1, i) and (j-1, j); minchange < 0, or 0 with i = j = 0 when no
 * improving move exists. */
typedef struct logo_move {
    uint32_t i;
    uint32_t j;
    int32_t minchange;
} logo_move;

typedef struct logo_stats {
    uint64_t moves;        /* 2-opt moves applied */
    uint64_t sweeps;       /* best-improvement sweeps evaluated */
    uint64_t pair_evals;   /* sweeps * (n-2)(n-3)/2 */
    uint64_t descents;     /* local-search descents run */
    uint64_t kicks;        /* perturbations applied */
    uint64_t accepted;     /* descents that improved the best tour */
    uint64_t start_length; /* length of the input tour */
    uint64_t final_length; /* length of the returned tour */
    double device_ms;      /* device time of the call (CUDA events) */
} logo_stats;

/* ILS perturbation kinds. */
#define LOGO_KICK_SEGMENT 0       /* reference kick: random segment reversal,
                                     src/solvers/ILSGlobalSolver.cpp:37-48 */
#define LOGO_KICK_DOUBLE_BRIDGE 1 /* double bridge with 3 uniform cuts
                                     (no reference counterpart) */

typedef struct logo_ctx logo_ctx;

/* ---- single instance ------------------------------------------------------ */

/* Creates a context for one instance on `device` and copies the coordinates
 * to it.  Replaces CUDASolver::init (src/solvers/CUDASolver.cpp:52-139). */
logo_status logo_ctx_create(int device, const logo_xy *coords, uint32_t n,
                            logo_ctx **out);

/* Frees the context.  Replaces CUDASolver::cleanCUDA
 * (src/solvers/CUDASolver.cpp:386-400).  NULL is accepted. */
logo_status logo_ctx_destroy(logo_ctx *ctx);

/* Text of the last error on this context (sticky until the next failing
 * call), or of the last failed logo_ctx_create on this thread when ctx is
 * NULL.  Never NULL. */
const char *logo_last_error(const logo_ctx *ctx);

/* One best-improvement sweep over `route` (n city ids): the best 2-opt move
 * or minchange = 0.  Replaces LocalSolver::optimizeStep / CUDASolver::
 * optimizeStep (src/solvers/localSolver.h:124-125,
 * src/solvers/CUDASolver.cpp:285-386). */
logo_status logo_best_move(logo_ctx *ctx, const uint32_t *route, logo_move *out);

/* 2-opt descent to a local optimum; route_inout is overwritten (on success
 * only) with the final tour.  max_moves = 0 means no limit.  Replaces
 * TwoOptLocalSolver::optimize (src/solvers/twoOptLocalSolver.cpp:22-64). */
logo_status logo_descend(logo_ctx *ctx, uint32_t *route_inout, uint64_t max_moves,
                         logo_stats *stats);

/* Iterated local search: descend, then `kicks` times {kick; descend; keep
 * the tour if strictly shorter than the best, else return to the best}.
 * route_inout receives the best tour.  Replaces
 * ILSGlobalSolverSequential::optimize
 * (src/solvers/ILSGlobalSolverSequential.cpp:60-100), whose stop rule needs
 * a known optimum, with an explicit kick count; kicks draw from SplitMix64
 * seeded with `seed` instead of rand(). */
logo_status logo_ils(logo_ctx *ctx, uint32_t *route_inout, uint32_t kicks,
                     uint64_t seed, int kick_kind, logo_stats *stats);

/* Tour length (routeLength, src/headers.h:170-189). */
logo_status logo_tour_length(logo_ctx *ctx, const uint32_t *route, uint64_t *length);

/* logo_descend that also records every applied move as (minchange, i, j)
 * int32 triples into move_log[0 .. 3*log_cap) -- the per-move report that
 * TwoOptLocalSolver::optimize prints when showLocalOptimizationInfo is set
 * (src/solvers/twoOptLocalSolver.cpp:56-65). */
logo_status logo_descend_trace(logo_ctx *ctx, uint32_t *route_inout, uint64_t max_moves,
                               int32_t *move_log, uint64_t log_cap, logo_stats *stats);

/* ---- allocation-free sweep ----------------------------------------------------- */

#define LOGO_NOALLOC_MAX_CITIES 65536u

/* No counterpart in the reference.  A best-improvement sweep for callers that
 * must not allocate device memory: callers that route every device byte
 * through their own pool allocator, and callers that cannot afford
 * cudaMalloc/cudaFree because those may synchronise the device.  All pointers
 * are device pointers owned by the caller: coords (n cities), route (n city
 * ids), out (one logo_move, written as logo_best_move would) and status_out
 * (optional; receives LOGO_OK, or LOGO_ERR_INVALID_ARG when route is not a
 * permutation of 0..n-1 or the coordinates are unusable).  Work is enqueued
 * on `stream` (a cudaStream_t; NULL = legacy default stream) and the call
 * returns without waiting.  coords must be 8-byte aligned (it is read as
 * (x, y) pairs: a cudaMalloc'd array, or an even element offset into one);
 * route, out and status_out 4-byte aligned; misaligned pointers are refused
 * with LOGO_ERR_INVALID_ARG before any work.  It allocates nothing: its working memory is a
 * fixed static device array of LOGO_NOALLOC_MAX_CITIES cities (1 MiB plus an
 * 8.25 KiB header) that every GPU loading the library holds until exit.
 * n above that maximum is rejected with LOGO_ERR_INVALID_ARG.  The first call
 * on each device looks up the array's device address (make it before any
 * stream capture; a device reset re-creates the array, and the first call
 * after it looks the address up again).  All calls share the array, so calls whose work overlaps
 * on the GPU race with each other; the caller must order them. */
logo_status logo_best_move_noalloc(const logo_xy *coords, const uint32_t *route, uint32_t n,
                                   logo_move *out, int32_t *status_out, void *stream);

/* ---- resident tour (no host copies between calls) --------------------------- */

/* Uploads a start tour that stays on the device. */
logo_status logo_set_route(logo_ctx *ctx, const uint32_t *route);
/* Downloads the resident tour. */
logo_status logo_get_route(logo_ctx *ctx, uint32_t *route);
/* Runs up to max_moves descent moves on the resident tour; stats->moves
 * receives how many were applied (fewer means a local optimum was reached). */
logo_status logo_descend_resident(logo_ctx *ctx, uint64_t max_moves, logo_stats *stats);
/* One sweep on the resident tour without applying the move. */
logo_status logo_sweep_resident(logo_ctx *ctx, logo_move *out);
/* Length of the resident tour. */
logo_status logo_length_resident(logo_ctx *ctx, uint64_t *length);
/* Waits for the context's stream. */
logo_status logo_sync(logo_ctx *ctx);

/* ---- stream-ordered primitives (enqueue only; no host synchronisation) ----- */

/* Starts a descent on the resident tour: clears the convergence flag and the
 * move counter; max_moves = 0 means no limit. */
logo_status logo_begin_descent(logo_ctx *ctx, uint64_t max_moves);
/* Enqueues one best-improvement sweep of the resident tour -- the kernel
 * launch of CUDASolver::executeKernel (src/solvers/CUDASolver.cpp:403-434)
 * with the argmin reduced on the device.  A no-op once converged. */
logo_status logo_enqueue_sweep(logo_ctx *ctx);
/* Enqueues the application of the last sweep's move on the device (the
 * rotate+reverse of src/solvers/twoOptLocalSolver.cpp:41-48), or sets the
 * convergence flag when the sweep found no improving move. */
logo_status logo_enqueue_apply(logo_ctx *ctx);
/* Waits for the stream and reports moves applied since logo_begin_descent
 * and whether the descent has converged. */
logo_status logo_get_progress(logo_ctx *ctx, uint64_t *moves, int *converged);

/* ---- batched solving (no reference counterpart) ------------------------------ */

#define LOGO_BATCH_MAX_N 4096u  /* largest instance of a batch (held in smem) */

/* One instance of a batch.  The caller owns both arrays; route is the start
 * tour on input and the best tour found on output. */
typedef struct logo_instance {
    const logo_xy *coords;
    uint32_t *route;
    uint32_t n;
    uint64_t seed; /* kick PRNG seed (SplitMix64 state) */
} logo_instance;

/* Tile shape of the batched kernel: rows per thread, threads per CTA (one
 * CTA per instance), columns per warp tile. */
typedef struct logo_batch_shape {
    int rows_per_thread;
    int threads_per_cta;
    int tile_cols;
} logo_batch_shape;

/* Start tours of a batch: the routes passed in, or tours built on the device
 * (the routes are then outputs only): nearest-neighbour tours equal to
 * logo_nn_tour from city 0, built by each instance's solving CTA, or
 * multiple-fragment tours equal to logo_mf_tour, built by one CTA per
 * instance in a launch before the solve (initRoute_KD_NN and
 * multipleFragment_KD, src/utils/kdtree_utils.c:279-301 and 56-242). */
#define LOGO_START_GIVEN 0
#define LOGO_START_NN 1
#define LOGO_START_MF 2

typedef struct logo_batch_opts {
    int device;
    uint32_t kicks;         /* ILS kicks per instance; 0 = descent only */
    int kick_kind;          /* LOGO_KICK_* */
    logo_batch_shape shape; /* all zero = use the tuned (or default) table */
    uint32_t ctas;          /* persistent CTAs; 0 = SMs x occupancy */
    int start;              /* LOGO_START_* */
} logo_batch_opts;

typedef struct logo_result {
    uint64_t start_length;
    uint64_t best_length;
    uint64_t moves;
    uint64_t sweeps;
    uint32_t kicks;
    uint32_t accepted;
    int32_t status; /* logo_status of this instance */
    uint32_t pad;
} logo_result;

typedef struct logo_batch logo_batch;

/* A reusable batch solver on `device` for up to max_count instances with at
 * most max_cities cities in total. */
logo_status logo_batch_create(int device, uint32_t max_count, uint64_t max_cities,
                              logo_batch **out);
logo_status logo_batch_destroy(logo_batch *b);
const char *logo_batch_last_error(const logo_batch *b);

/* Solves every instance independently -- descent, then opts->kicks ILS
 * iterations, each exactly as logo_ils would -- in one persistent launch per
 * tile shape used: instances are handed out longest first from a device work
 * queue, one CTA per instance with the whole instance in shared memory.
 * Every instance needs 3 <= n <= LOGO_BATCH_MAX_N.  device_ms (optional)
 * receives the device time of the solve. */
logo_status logo_batch_run(logo_batch *b, const logo_instance *inst, uint32_t count,
                           const logo_batch_opts *opts, logo_result *results,
                           double *device_ms);

/* Multi-start ILS (ILSGlobalSolverMT, src/solvers/ILSGlobalSolverMT.cpp:86-195,
 * with its --comm sharing when share != 0): `replicas` copies of one instance
 * (3 <= n <= LOGO_BATCH_MAX_N), replica k kicked from seed + k, all solved in
 * one persistent launch, one CTA per replica.  Without share every replica
 * equals logo_ils with its seed.  With share, a replica whose descent does not
 * beat its own best continues from the best tour any replica has published
 * (the reference's threads do the same with the global best), and it
 * publishes its own best whenever that beats the group's; publishing never
 * waits (a replica that finds another one publishing offers again after its
 * next descent), so shared runs depend on timing.  route: start tour in, the
 * best replica's tour out; results (optional) receives one entry per replica,
 * best (optional) the replica returned; b needs max_count >= replicas and
 * max_cities >= n * replicas. */
logo_status logo_batch_multistart(logo_batch *b, const logo_xy *coords, uint32_t n,
                                  uint32_t *route, uint32_t replicas, uint64_t seed, int share,
                                  const logo_batch_opts *opts, logo_result *results,
                                  uint32_t *best, double *device_ms);

/* One-shot logo_batch_create + logo_batch_run + logo_batch_destroy. */
logo_status logo_batch_solve(const logo_instance *inst, uint32_t count,
                             const logo_batch_opts *opts, logo_result *results,
                             double *device_ms);

/* Autotuner: times every compiled tile shape on the given sample per size
 * bucket (n < 128, < 384, < 1024, < 2048, <= 4096) and installs the fastest
 * as this batch's table; results are also merged into the JSON file at
 * cache_path (keyed by GPU name and bucket) when it is not NULL.  With
 * reuse != 0 a matching cache entry is loaded instead of timing. */
logo_status logo_batch_autotune(logo_batch *b, const logo_instance *sample, uint32_t count,
                                uint32_t kicks, int kick_kind, const char *cache_path,
                                int reuse);
/* The shape used for instances of size n. */
logo_status logo_batch_shape_for(const logo_batch *b, uint32_t n, logo_batch_shape *out);

/* ---- serving: continuous batching of requests (no reference counterpart) ----- */

typedef struct logo_server logo_server;

typedef struct logo_server_opts {
    int device;
    uint64_t mem_budget;    /* device bytes for resident requests; 0 = 2 GiB */
    uint32_t max_slots;     /* requests with n <= LOGO_BATCH_MAX_N in flight; 0 = SMs x occupancy */
    uint32_t max_large;     /* larger requests in flight; 0 = 2 */
    uint32_t kicks;         /* ILS kicks per request after its first descent */
    int kick_kind;          /* LOGO_KICK_* */
    uint64_t quantum_pairs; /* pair evaluations per request per round; 0 = 2e7 */
    uint32_t max_pending;   /* submitted but not admitted; 0 = 1,000,000 */
} logo_server_opts;

typedef struct logo_request_info {
    uint64_t start_length;
    uint64_t best_length;
    uint64_t moves;
    uint64_t sweeps;
    uint32_t n;
    uint32_t kicks;
    uint32_t accepted;
    int32_t status;    /* logo_status of this request */
    double queue_ms;   /* submit -> admitted to the device */
    double latency_ms; /* submit -> result available */
} logo_request_info;

typedef struct logo_server_stats {
    uint64_t submitted, admitted, completed, failed;
    uint64_t pending, running_small, running_large;
    uint64_t rounds;
    double round_device_ms; /* device time of all rounds */
    uint64_t mem_in_use, mem_budget;
} logo_server_stats;

/* Starts a server: a scheduler thread that admits submitted requests while
 * the device-memory budget and slots allow, keeps their tours resident on the
 * device and advances all admitted small requests together in rounds of
 * bounded work (continuous batching: a request that arrives while others run
 * joins the next round).  Requests with n > LOGO_BATCH_MAX_N run concurrently
 * through the single-instance path.  Every request is solved exactly as
 * logo_ils would (descent, then `kicks` kicks with accept/revert), so its
 * result does not depend on what else is in flight. */
logo_status logo_server_create(const logo_server_opts *opts, logo_server **out);
/* Queues a request (inputs are copied; route is the start tour).  Thread
 * safe.  BUSY when max_pending requests are already waiting. */
logo_status logo_server_submit(logo_server *s, const logo_xy *coords, uint32_t n,
                               const uint32_t *route, uint64_t seed, uint64_t *id);
/* BUSY while the request is queued or running; otherwise copies the best
 * tour to route_out (n entries, may be NULL), fills info and forgets the
 * request (NOT_FOUND afterwards).  Returns the request's own status. */
logo_status logo_server_poll(logo_server *s, uint64_t id, uint32_t *route_out,
                             logo_request_info *info);
/* logo_server_poll that waits up to timeout_ms for completion. */
logo_status logo_server_wait(logo_server *s, uint64_t id, uint32_t timeout_ms,
                             uint32_t *route_out, logo_request_info *info);
logo_status logo_server_get_stats(logo_server *s, logo_server_stats *out);
/* Stops the server; running requests are finished, queued ones dropped. */
logo_status logo_server_destroy(logo_server *s);
const char *logo_server_last_error(const logo_server *s);

/* ---- host-side entry points around the path (no GPU needed) -------------------- */

/* Reads a TSPLIB NODE_COORD_SECTION file into coords[0..n) (float x, y, as
 * readFileCoords does, src/utils/tsp_loader.c:49-162).  Header lines are
 * parsed by keyword (the reference skips a fixed 3 lines, :72-94).  With
 * coords = NULL only *n is returned.  NOT_FOUND if the file cannot be
 * opened, INVALID_ARG if it is malformed or larger than cap. */
logo_status logo_read_tsplib(const char *path, logo_xy *coords, uint32_t cap, uint32_t *n);

/* Nearest-neighbour start tour from city `start` (initRoute_KD_NN,
 * src/utils/kdtree_utils.c:279-301, which starts at city 0): repeatedly the
 * nearest unvisited city by double-precision Euclidean distance, ties to the
 * lowest id.  Unlike the reference's kd-tree, duplicate points are kept. */
logo_status logo_nn_tour(const logo_xy *coords, uint32_t n, uint32_t start, uint32_t *route);

/* TSPLIB EDGE_WEIGHT_TYPE values reported by logo_tsplib_info.  The engine
 * computes EUC_2D nint distances, as the reference does for every file it
 * reads (readFileCoords, src/utils/tsp_loader.c:49-162, only loads the
 * coordinates); the type lets a caller refuse files meant for another metric. */
#define LOGO_EWT_EUC_2D 0
#define LOGO_EWT_CEIL_2D 1
#define LOGO_EWT_ATT 2
#define LOGO_EWT_GEO 3
#define LOGO_EWT_OTHER 4
/* Header of a TSPLIB file: DIMENSION into *n (optional) and EDGE_WEIGHT_TYPE
 * into *edge_weight_type (optional; EUC_2D when the header has none).
 * NOT_FOUND if the file cannot be opened, INVALID_ARG without a valid
 * DIMENSION.  No counterpart in the reference. */
logo_status logo_tsplib_info(const char *path, uint32_t *n, int *edge_weight_type);

/* Reads a tour (routeInitFromFile, src/utils/common.c:109-128, which reads
 * a bare list of 1-based ids): either that list or a TSPLIB .tour file
 * (NAME/TYPE/DIMENSION header, TOUR_SECTION, ids, -1, EOF).  The ids must be
 * a permutation of 1..n (and match DIMENSION when given); route receives them
 * 0-based.  With route = NULL only *n is returned.  NOT_FOUND if the file
 * cannot be opened, INVALID_ARG if it is malformed or n > cap. */
logo_status logo_read_tour(const char *path, uint32_t *route, uint32_t cap, uint32_t *n);

/* Writes a tour as 1-based ids (saveRouteToAFile, src/utils/common.c:144-192):
 * with tsplib_header != 0 as a TSPLIB .tour file (NAME `name`, TYPE TOUR,
 * DIMENSION, TOUR_SECTION, ids, -1, EOF), else as the reference's bare list
 * (which its reader accepts).  INVALID_ARG unless route is a permutation of
 * 0..n-1; NOT_FOUND if the file cannot be written. */
logo_status logo_write_tour(const char *path, const uint32_t *route, uint32_t n,
                            const char *name, int tsplib_header);

/* Multiple-fragment (greedy edge) start tour (multipleFragment_KD,
 * src/utils/kdtree_utils.c:56-242, the reference's --init mf): repeatedly the
 * shortest nint edge from a city to its nearest city of degree < 2 outside
 * its own fragment, taken in the reference's priority-queue order so that
 * equal lengths are broken the same way; the path is listed from city 0 as
 * the reference lists it.  Neighbour searches use a uniform grid, ties to the
 * lowest id (the reference's kd-tree breaks exact distance ties by traversal
 * order and mishandles duplicate points). */
logo_status logo_mf_tour(const logo_xy *coords, uint32_t n, uint32_t *route);

/* The k nearest other cities of every city (1 <= k <= 64): out[v*k + j],
 * nearest first, by squared distance in double with ties to the lower id;
 * with fewer than k other cities the remaining slots repeat the last one
 * found (v itself when n == 1).  The candidate lists of LOGO_SEARCH_NEIGHBOUR
 * (no reference counterpart).  From 20,000 cities this and logo_mf_tour
 * spread their per-city queries over up to 16 host threads (the environment
 * variable LOGO_HOST_THREADS sets the count); results do not depend on it. */
logo_status logo_neighbours(const logo_xy *coords, uint32_t n, uint32_t k, uint32_t *out);

/* Seeded random start tour (routeInit with ROUTE_INIT_SHUFFLE,
 * src/utils/construction.c:129-137, which uses random_shuffle on rand()):
 * Fisher-Yates driven by SplitMix64. */
logo_status logo_random_tour(uint32_t n, uint64_t seed, uint32_t *route);

/* 1 if route is a permutation of 0..n-1 with n >= 3 (checkTour,
 * src/utils/construction.c:152-183, which exit()s instead), else 0. */
int logo_check_tour(const uint32_t *route, uint32_t n);

/* ---- introspection ------------------------------------------------------------- */

typedef struct logo_ctx_info {
    uint32_t n;
    int device;
    int rows_per_thread;  /* sweep tile shape chosen for this n */
    int warps_per_cta;
    uint32_t tile_cols;
    uint32_t tiles;       /* CTAs per sweep */
    float filter_margin;  /* bound on |exact - approximate delta| */
    uint32_t graph_steps; /* sweep+apply steps per graph launch */
    int variant;          /* LOGO_SWEEP_* */
    int descent_mode;     /* LOGO_DESCENT_* in use */
    int cooperative_ctas; /* CTAs of the cooperative descent; 0 if unavailable */
    uint64_t host_waits;  /* times this context's calls have waited on the device so far
                             (one logo_ils call: a fixed handful, whatever the kick count) */
    int route_io;         /* LOGO_ROUTE_IO_COPY or LOGO_ROUTE_IO_DIRECT in use */
    int search;           /* LOGO_SEARCH_* */
    uint32_t search_neighbours; /* neighbour-list length of LOGO_SEARCH_NEIGHBOUR */
    uint32_t pad0;
} logo_ctx_info;

logo_status logo_ctx_get_info(const logo_ctx *ctx, logo_ctx_info *info);

/* Overrides the sweep tile shape (rows per thread, warps per CTA, columns per
 * tile); used by the autotuner.  Invalid shapes return INVALID_ARG. */
logo_status logo_ctx_set_shape(logo_ctx *ctx, int rows_per_thread, int warps_per_cta,
                               uint32_t tile_cols);

/* How a descent is driven; all modes return identical moves.
 * LOGO_DESCENT_AUTO (default): COOPERATIVE where available, else GRAPH.
 * LOGO_DESCENT_GRAPH: captured CUDA graphs of (sweep, gather) launches,
 *   replayed until the device convergence flag is set.
 * LOGO_DESCENT_COOPERATIVE: one cooperative persistent launch per descent
 *   (tours of 8 to 6,144 cities, held in every CTA's shared memory; one
 *   grid barrier per move).  No counterpart in the reference, whose descent is a
 *   host loop over optimizeStep (src/solvers/twoOptLocalSolver.cpp:22-64). */
#define LOGO_DESCENT_AUTO 0
#define LOGO_DESCENT_GRAPH 1
#define LOGO_DESCENT_COOPERATIVE 2
/* INVALID_ARG for an unknown mode, or COOPERATIVE where it is unavailable. */
logo_status logo_ctx_set_descent_mode(logo_ctx *ctx, int mode);

/* How the route buffers of logo_descend, logo_ils, logo_best_move,
 * logo_tour_length, logo_set_route and logo_get_route reach the device; both
 * give identical results.
 * LOGO_ROUTE_IO_AUTO (default): DIRECT where the device can read and write
 *   pageable host memory (cudaDevAttrPageableMemoryAccess, e.g. a coherent
 *   CPU-GPU link), else COPY.
 * LOGO_ROUTE_IO_COPY: cudaMemcpyAsync from and to the caller's buffer.
 * LOGO_ROUTE_IO_DIRECT: the load and store kernels read and write the
 *   caller's buffer in place (one wait per logo_descend call instead of two).
 * Route buffers must then be valid for n uint32_t, as for a copy. */
#define LOGO_ROUTE_IO_AUTO 0
#define LOGO_ROUTE_IO_COPY 1
#define LOGO_ROUTE_IO_DIRECT 2
/* INVALID_ARG for an unknown mode, or DIRECT where the device cannot reach
 * pageable host memory. */
logo_status logo_ctx_set_route_io(logo_ctx *ctx, int mode);

/* Which moves a descent (logo_descend, logo_descend_resident, the descents of
 * logo_ils) applies.
 * LOGO_SEARCH_EXHAUSTIVE (default): the best of all (n-2)(n-3)/2 pairs each
 *   step -- the reference's best improvement (CPUSolver::optimizeStep,
 *   src/solvers/cpuSolver.cpp:104-146), bit-exact.
 * LOGO_SEARCH_NEIGHBOUR: first the best of the 2-opt moves that create an
 *   edge from a city to one of its `neighbours` nearest cities (2 x
 *   neighbours x n candidate pairs per step, lowest (delta, i, j) first),
 *   until none improves; then full sweeps as above to a local optimum of
 *   the whole pair set.  The end point is a 2-opt local optimum, reached
 *   along another path than the reference's, in far fewer pair evaluations
 *   at large n (no counterpart in the reference).  The neighbour phase of
 *   a descent is one cooperative launch where the device allows it (inside
 *   logo_ils a cooperative kernel node of its graph; graph launches with
 *   LOGO_DESCENT_GRAPH); the full sweeps after it use graph launches.
 * LOGO_SEARCH_NEIGHBOUR_OROPT: as NEIGHBOUR, and each step also weighs the
 *   Or-opt moves that create an edge to a listed neighbour: a segment of 1
 *   to 3 cities moved, in order or reversed, into another gap of the tour
 *   (neither side of the closing edge is cut); the lowest delta wins, ties
 *   to the 2-opt move, then to shorter and unreversed segments, then to the
 *   lower (segment start, gap).
 * neighbours: 1..16, 0 = 8.  INVALID_ARG for an unknown mode or list
 * length. */
/* The start tour of the context's instance built on the device, written to
 * route (n entries): LOGO_START_NN (equal to logo_nn_tour from city 0) or
 * LOGO_START_MF (equal to logo_mf_tour), by one CTA as in the batched launch;
 * n <= LOGO_BATCH_MAX_N, else INVALID_ARG (the host builders then).  The
 * resident tour is not changed. */
logo_status logo_start_tour(logo_ctx *ctx, int kind, uint32_t *route);

#define LOGO_SEARCH_EXHAUSTIVE 0
#define LOGO_SEARCH_NEIGHBOUR 1
#define LOGO_SEARCH_NEIGHBOUR_OROPT 2
logo_status logo_ctx_set_search(logo_ctx *ctx, int mode, uint32_t neighbours);

/* Sweep kernel variants; all return identical moves (the default depends on
 * n, see logo_ctx_info.variant).
 * LOGO_SWEEP_MUFU: pairs are screened with approximate square roots (MUFU)
 *   and an error margin.
 * Values 1-3 are retired (a paired-f32x2 MUFU screen and two plain
 *   squared-distance screens that no size chose; LOGO_ERR_INVALID_ARG).
 * LOGO_SWEEP_FUSED: two-stage squared screen with the window threshold
 *   folded into the sum of squares: d(i, c) for every pair (FADD2/FFMA2, two
 *   rows at a time), d(i-1, c-1) only where that passes; threads share the
 *   best delta found so far within a sweep.
 * LOGO_SWEEP_LOCAL: the test on d(i, c) expanded in coordinates relative to
 *   the tile's first row, |q|^2 - 2 r.q against a per-row threshold with a
 *   proven rounding margin (two FFMA per pair), then the fused screen's
 *   remaining stages.
 * LOGO_SWEEP_BOXED: three launches per sweep.  (1) The bounding box and
 *   largest edge of every 32-city window; (2) a tile filter that keeps only
 *   tiles with a (32-row window, 32-column window) pair whose box distance
 *   lets some pair be chosen; (3) a persistent sweep over the kept tiles
 *   that tests each thread's rows against each window's box with the live
 *   best delta and evaluates what is left pair by pair, one lane per column
 *   (or, on tiles where most rows are open, with the local screen).  Tile
 *   widths must be multiples of 32 up to 1024. */
#define LOGO_SWEEP_MUFU 0
#define LOGO_SWEEP_FUSED 4
#define LOGO_SWEEP_LOCAL 5
#define LOGO_SWEEP_BOXED 6
/* Selects variant and tile shape together (logo_ctx_set_shape keeps the
 * variant).  Shapes per variant: MUFU (R,NW) in {(2,2),(2,4),(4,2),(4,4),
 * (4,8),(8,4),(8,8),(16,4)}; FUSED {(4,2),(4,4),(4,8),(8,2),(8,4),(8,8),(16,4)};
 * LOCAL and BOXED {(4,2),(4,4),(4,8),(8,4),(8,8),(16,4)}; 16 <= cols <= 4096
 * (BOXED: a multiple of 32, at most 1024). */
logo_status logo_ctx_set_kernel(logo_ctx *ctx, int variant, int rows_per_thread,
                                int warps_per_cta, uint32_t tile_cols);

/* The CUDA stream (cudaStream_t) the context launches on, for callers that
 * time or order work against it. */
void *logo_ctx_stream(logo_ctx *ctx);

/* Library version string. */
const char *logo_version(void);

/* Test hook for failure detection (no counterpart in the reference): runs
 * two device waits that nothing will satisfy -- an mbarrier expecting bytes
 * that no copy delivers (the sweeps' staging wait) and the cooperative
 * descent's grid barrier with one of two CTAs missing -- and returns the
 * status bits each left (1 = gave up after its 2 s budget) and the time the
 * pair took.  Nothing faults or hangs; the device stays usable. */
logo_status logo_diag_wait_limits(int device, uint32_t *mbarrier_status,
                                  uint32_t *barrier_status, double *waited_ms);

/* Test hook for the host side of a device timeout (no counterpart in the
 * reference): sets the timeout bit in the context's device status word, as a
 * sweep wait or the cooperative grid barrier does when it gives up, without
 * any wait running out.  The next call that reads the status returns
 * LOGO_ERR_TIMEOUT and every later call on the context LOGO_ERR_DEVICE_FAULT
 * (a context whose device wait timed out is never used again; destroy it). */
logo_status logo_diag_flag_timeout(logo_ctx *ctx);

/* Self-check of the sweep's exactness argument: the largest relative error of
 * the device's approximate square root over every positive normal binary32
 * input, against the correctly rounded root.  The sweep's filter margin
 * assumes it is at most 2^-20.  No reference counterpart. */
logo_status logo_diag_sqrt_error(int device, double *max_rel_err);

#ifdef __cplusplus
}
#endif
#endif /* LOGO_GPU_H */
