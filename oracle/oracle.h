/*
 * CPU oracle for the 2-opt hot path of the LOGO TSP solver.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; it is the checker that the CUDA path is compared against
 * (tests/, __graft_entry__.smoke() and the cpu_baseline / reference legs of
 * bench.py).
 *
 * Each function restates one piece of the reference's algorithm in plain C and
 * cites the reference file:line it follows (paths relative to the reference
 * project root).  The distance is the reference's per-edge EUC_2D nint,
 *     (int)(sqrtf(dx*dx + dy*dy) + 0.5f)
 * (src/cuda/cuda_common.h:33-40, src/headers.h:126-133), evaluated in IEEE
 * binary32 with no FMA contraction (the file is compiled with
 * -ffp-contract=off) and a correctly rounded sqrtf.
 *
 * Pinning: the reference ships no tests or golden vectors for this path.  The
 * oracle is pinned against the reference's own sources compiled here
 * (oracle/build_ref.sh -> oracle/_ref/): move application and descent
 * (TwoOptLocalSolver::optimize), tour length (routeLength), the segment
 * reversal kick (ILSGlobalSolver::kick), the ILS accept/revert loop and the
 * kd-tree nearest-neighbour start tour all run from the reference's code in
 * that harness, and tests/test_oracle_ref.py compares them with this file.
 *
 * Coordinates are AoS pairs (x0,y0,x1,y1,...) like city_coords
 * (src/defs.h:173-178); routes are uint32 city ids (ROUTE_DATA_TYPE,
 * src/defs.h:22).
 */
#ifndef LOGO_ORACLE_H
#define LOGO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-edge EUC_2D nint distance, src/cuda/cuda_common.h:33-40. */
int32_t lo_dist(float ax, float ay, float bx, float by);

/* SplitMix64 (Steele, Lea, Flood, OOPSLA 2014): the project PRNG that replaces
 * the reference's wall-clock-seeded rand() (src/utils/common.c:253-259). */
uint64_t lo_splitmix64(uint64_t *state);
/* Uniform integer in [0, n): high 32 bits of the next output, scaled by n. */
uint32_t lo_uniform(uint64_t *state, uint32_t n);

/* Packed argmin key: ((delta + 2^22) << 42) | (i << 21) | j.  Unsigned
 * comparison orders by delta, then i, then j -- the reference CPU order
 * (src/solvers/cpuSolver.cpp:188-230: i ascending, j ascending, strict <). */
uint64_t lo_pack_key(int32_t delta, uint32_t i, uint32_t j);

/* One best-improvement sweep: CPUSolver::optimizeStep
 * (src/solvers/cpuSolver.cpp:143-230) with the per-edge nint distance.
 * Pairs 1 <= i < j <= n-2 over tour positions; reports the move as (i, j+1)
 * like the reference (out.j = j + 1).  Returns 1 and fills delta/i/j when an
 * improving move (delta < 0) exists, else 0 (delta = 0). */
int lo_best_move(const float *xy, const uint32_t *route, uint32_t n,
                 int32_t *delta, uint32_t *mi, uint32_t *mj);

/* Same sweep restricted to rows i in [row_lo, row_hi) -- used to time a
 * bounded sample of a sweep.  Returns the packed key or UINT64_MAX. */
uint64_t lo_best_move_rows(const float *xy, const uint32_t *route, uint32_t n,
                           uint32_t row_lo, uint32_t row_hi);

/* Multi-threaded sweep over `threads` pthreads, splitting the row range like
 * CPUMTSolver::optimizeStep (src/solvers/cpuMTSolver.cpp:79-158).  Same result
 * as lo_best_move.  Rows [row_lo, row_hi) (row_hi = 0 means all rows). */
uint64_t lo_best_move_mt(const float *xy, const uint32_t *route, uint32_t n,
                         uint32_t row_lo, uint32_t row_hi, int threads);

/* Move application, src/solvers/twoOptLocalSolver.cpp:41-48:
 * swap so bi > bj; rotate(begin, begin+bj, end); reverse(begin+(bi-bj), end).
 * tmp must hold n entries. */
void lo_apply_move(uint32_t *route, uint32_t n, uint32_t mi, uint32_t mj,
                   uint32_t *tmp);

/* Tour length, routeLength (src/headers.h:170-189): sum of per-edge nint
 * distances including the closing edge. */
uint64_t lo_tour_length(const float *xy, const uint32_t *route, uint32_t n);

/* 2-opt descent, TwoOptLocalSolver::optimize
 * (src/solvers/twoOptLocalSolver.cpp:22-64): step + apply until no improving
 * move.  If move_log is non-NULL it receives (delta, i, j) triples for up to
 * log_cap moves.  Returns the number of moves, or -1 if max_moves was hit. */
int64_t lo_descend(const float *xy, uint32_t *route, uint32_t n,
                   uint64_t max_moves, int32_t *move_log, uint64_t log_cap);
/* The same descent with every sweep split over `threads` pthreads (same moves). */
int64_t lo_descend_mt(const float *xy, uint32_t *route, uint32_t n,
                      uint64_t max_moves, int32_t *move_log, uint64_t log_cap,
                      int threads);

/* Kick kinds for the ILS perturbation. */
#define LO_KICK_SEGMENT 0       /* reference kick, ILSGlobalSolver.cpp:37-48 */
#define LO_KICK_DOUBLE_BRIDGE 1 /* new: 3 cuts, A B C D -> A C B D          */

/* ILSGlobalSolver::kick (src/solvers/ILSGlobalSolver.cpp:37-48) with rand()
 * replaced by lo_uniform: a, b uniform in [0,n), sorted, rotate by a, reverse
 * [b-a, n). */
void lo_kick_segment(uint32_t *route, uint32_t n, uint64_t *rng, uint32_t *tmp);

/* Double-bridge (no reference counterpart): three cut points c = 1 +
 * uniform(n-1), sorted p1 <= p2 <= p3; new = old[0,p1) old[p2,p3) old[p1,p2)
 * old[p3,n). */
void lo_kick_double_bridge(uint32_t *route, uint32_t n, uint64_t *rng,
                           uint32_t *tmp);

typedef struct {
    uint64_t moves;        /* 2-opt moves applied over all descents */
    uint64_t descents;     /* kicks + 1 */
    uint64_t accepted;     /* descents whose result became the new best */
    uint64_t start_length; /* length of the input tour */
    uint64_t best_length;  /* length of the returned tour */
} lo_ils_stats;

/* ILS, ILSGlobalSolverSequential::optimize
 * (src/solvers/ILSGlobalSolverSequential.cpp:60-100) driven by an explicit
 * kick count: descend; accept if strictly shorter than the best, else revert
 * to the best; kick; ... (kicks + 1 descents).  The route is overwritten with
 * the best tour.  Returns 0, or -1 if a descent exceeded max_moves. */
int lo_ils(const float *xy, uint32_t *route, uint32_t n, uint32_t kicks,
           uint64_t seed, int kick_kind, uint64_t max_moves_per_descent,
           lo_ils_stats *stats);
/* The same ILS with every sweep split over `threads` pthreads (same result). */
int lo_ils_mt(const float *xy, uint32_t *route, uint32_t n, uint32_t kicks,
              uint64_t seed, int kick_kind, uint64_t max_moves_per_descent,
              lo_ils_stats *stats, int threads);

/* Neighbour-list search (LOGO_SEARCH_NEIGHBOUR; no reference counterpart):
 * lo_knn writes the k nearest other cities of every city (squared double
 * distance, lower id on ties, out[v*k + j] nearest first; fewer than k other
 * cities repeat the last one found, or v itself).  lo_descend_nbr first
 * applies the best improving move among the pairs that create an edge from
 * a city to one of its listed neighbours until none improves, then full
 * best-improvement sweeps (as lo_descend) to a local optimum; moves of both
 * phases count towards max_moves, *nbr_moves gets the first phase's.
 * lo_ils_nbr is lo_ils_mt with those descents.  With oropt the neighbour
 * phase also weighs Or-opt moves (segments of 1-3 cities moved, in order or
 * reversed, next to a listed neighbour; LOGO_SEARCH_NEIGHBOUR_OROPT). */
int lo_knn(const float *xy, uint32_t n, uint32_t k, uint32_t *out);
int64_t lo_descend_nbr(const float *xy, uint32_t *route, uint32_t n, const uint32_t *nbr,
                       uint32_t k, uint64_t max_moves, int threads, uint64_t *nbr_moves,
                       int oropt);
int lo_nbr_step(const float *xy, const uint32_t *route, uint32_t n, const uint32_t *nbr,
                uint32_t k, int oropt, int32_t *delta, int32_t *slot, uint32_t *i, uint32_t *j);
int lo_ils_nbr(const float *xy, uint32_t *route, uint32_t n, uint32_t kicks, uint64_t seed,
               int kick_kind, uint64_t max_moves_per_descent, lo_ils_stats *stats,
               int threads, const uint32_t *nbr, uint32_t k, int oropt);

/* Nearest-neighbour start tour, initRoute_KD_NN
 * (src/utils/kdtree_utils.c:279-301): start at city 0, repeatedly go to the
 * nearest unvisited city by squared distance in double; ties go to the lowest
 * city id.  Returns the number of exact distance ties met (0 means the
 * tour does not depend on the tie rule). */
uint64_t lo_nn_tour(const float *xy, uint32_t n, uint32_t *route);

/* Permutation check, checkTour (src/utils/construction.c:152-183).
 * Returns 1 if route is a permutation of 0..n-1. */
int lo_check_tour(const uint32_t *route, uint32_t n);

/* Batch of independent ILS runs over `threads` pthreads, one instance per
 * thread at a time (the CPU comparison for batched solving).  Instance k has
 * coordinates xy + 2*offsets[k], n = ns[k], its route in routes + offsets[k]
 * and seed seeds[k].  best_lengths[k] receives the final length. */
int lo_ils_batch(const float *xy, uint32_t *routes, const uint64_t *offsets,
                 const uint32_t *ns, const uint64_t *seeds, uint32_t count,
                 uint32_t kicks, int kick_kind, int threads,
                 uint64_t *best_lengths, uint64_t *moves);

#ifdef __cplusplus
}
#endif
#endif
