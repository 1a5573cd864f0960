/*
 * CPU oracle for the 2-opt hot path -- TEST INFRASTRUCTURE ONLY (see
 * oracle.h).  Compiled with -O3 -ffp-contract=off -fno-math-errno: no FMA
 * contraction, IEEE binary32 arithmetic, correctly rounded sqrtf.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* src/cuda/cuda_common.h:33-40 and src/headers.h:126-133:
 * (int)(sqrtf(dx*dx + dy*dy) + 0.5f). */
int32_t lo_dist(float ax, float ay, float bx, float by)
{
    float dx = ax - bx;
    float dy = ay - by;
    float s = dx * dx + dy * dy;
    return (int32_t)(sqrtf(s) + 0.5f);
}

uint64_t lo_splitmix64(uint64_t *state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint32_t lo_uniform(uint64_t *state, uint32_t n)
{
    uint64_t hi = lo_splitmix64(state) >> 32;
    return (uint32_t)((hi * (uint64_t)n) >> 32);
}

uint64_t lo_pack_key(int32_t delta, uint32_t i, uint32_t j)
{
    return ((uint64_t)(uint32_t)(delta + (1 << 22)) << 42) |
           ((uint64_t)i << 21) | (uint64_t)j;
}

/* ------------------------------------------------------------------------ */
/* Sweep                                                                      */
/* ------------------------------------------------------------------------ */

/* Tour-ordered coordinates and incoming edge lengths, the USE_ORDERED_COORDS
 * gather of src/solvers/cpuSolver.cpp:151-163 plus const1 of :190. */
typedef struct {
    float *x, *y;
    int32_t *e; /* e[k] = d(k-1, k) for k >= 1; e[0] = closing edge */
    uint32_t n;
} ordered_t;

static int ordered_init(ordered_t *o, const float *xy, const uint32_t *route,
                        uint32_t n)
{
    o->n = n;
    o->x = (float *)malloc(sizeof(float) * (n + 1));
    o->y = (float *)malloc(sizeof(float) * (n + 1));
    o->e = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
    if (!o->x || !o->y || !o->e)
        return -1;
    for (uint32_t k = 0; k < n; k++) {
        o->x[k] = xy[2 * (size_t)route[k]];
        o->y[k] = xy[2 * (size_t)route[k] + 1];
    }
    for (uint32_t k = 1; k < n; k++)
        o->e[k] = lo_dist(o->x[k - 1], o->y[k - 1], o->x[k], o->y[k]);
    o->e[0] = n ? lo_dist(o->x[n - 1], o->y[n - 1], o->x[0], o->y[0]) : 0;
    return 0;
}

static void ordered_free(ordered_t *o)
{
    free(o->x);
    free(o->y);
    free(o->e);
}

/* Rows i in [lo, hi) of the pair triangle 1 <= i < j <= n-2, written with
 * column c = j + 1 in [i+2, n-1]:
 *   delta(i, c) = d(i, c) + d(i-1, c-1) - e[i] - e[c]
 * which is the reference's change(i, j) with the reported j+1
 * (src/solvers/cpuSolver.cpp:188-230).  The loop order is the reference's
 * (i ascending, then j ascending, strict <), so ties resolve to the lowest
 * (i, j).  Each distance d(i, c) is computed once per row and reused as
 * d(i-1, c-1) by the next row. */
static uint64_t sweep_rows(const ordered_t *o, uint32_t lo, uint32_t hi,
                           int32_t *prev, int32_t *cur, int32_t *dl)
{
    const uint32_t n = o->n;
    const float *X = o->x, *Y = o->y;
    const int32_t *E = o->e;
    uint64_t best = UINT64_MAX;
    int32_t bestd = 0;
    if (n < 4)
        return best;
    if (hi > n - 2)
        hi = n - 2;
    if (lo < 1)
        lo = 1;
    if (lo >= hi)
        return best;
    /* prev[c] = d(lo-1, c) for c in [lo+1, n-2] */
    {
        float ax = X[lo - 1], ay = Y[lo - 1];
        for (uint32_t c = lo + 1; c < n - 1; c++)
            prev[c] = lo_dist(ax, ay, X[c], Y[c]);
    }
    for (uint32_t i = lo; i < hi; i++) {
        const float ax = X[i], ay = Y[i];
        const int32_t ei = E[i];
        for (uint32_t c = i + 2; c < n; c++)
            cur[c] = lo_dist(ax, ay, X[c], Y[c]);
        int32_t rowmin = 0;
        for (uint32_t c = i + 2; c < n; c++) {
            int32_t v = cur[c] + prev[c - 1] - ei - E[c];
            dl[c] = v;
            rowmin = v < rowmin ? v : rowmin;
        }
        if (rowmin < bestd) {
            for (uint32_t c = i + 2; c < n; c++) {
                if (dl[c] == rowmin) {
                    bestd = rowmin;
                    best = lo_pack_key(rowmin, i, c);
                    break;
                }
            }
        }
        int32_t *t = prev;
        prev = cur;
        cur = t;
    }
    return best;
}

static uint64_t sweep_alloc_rows(const ordered_t *o, uint32_t lo, uint32_t hi)
{
    uint32_t n = o->n;
    int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(n + 1));
    if (!buf)
        return UINT64_MAX;
    uint64_t k = sweep_rows(o, lo, hi, buf, buf + (n + 1), buf + 2 * (n + 1));
    free(buf);
    return k;
}

static void unpack_key(uint64_t key, int32_t *delta, uint32_t *i, uint32_t *j)
{
    *delta = (int32_t)(key >> 42) - (1 << 22);
    *i = (uint32_t)((key >> 21) & 0x1FFFFF);
    *j = (uint32_t)(key & 0x1FFFFF);
}

int lo_best_move(const float *xy, const uint32_t *route, uint32_t n,
                 int32_t *delta, uint32_t *mi, uint32_t *mj)
{
    ordered_t o;
    *delta = 0;
    *mi = 0;
    *mj = 0;
    if (ordered_init(&o, xy, route, n)) {
        ordered_free(&o);
        return -1;
    }
    uint64_t key = sweep_alloc_rows(&o, 1, n);
    ordered_free(&o);
    if (key == UINT64_MAX)
        return 0;
    unpack_key(key, delta, mi, mj);
    return 1;
}

uint64_t lo_best_move_rows(const float *xy, const uint32_t *route, uint32_t n,
                           uint32_t row_lo, uint32_t row_hi)
{
    ordered_t o;
    if (ordered_init(&o, xy, route, n)) {
        ordered_free(&o);
        return UINT64_MAX;
    }
    uint64_t key = sweep_alloc_rows(&o, row_lo, row_hi ? row_hi : n);
    ordered_free(&o);
    return key;
}

/* Parallel sweep: blocks of rows handed out dynamically to pthreads; the
 * per-thread keys reduce with an unsigned min, which keeps the lowest-(i, j)
 * rule.  The reference splits the triangle's rows statically over
 * maxCoresCPU threads (src/solvers/cpuMTSolver.cpp:109-148). */
typedef struct {
    const ordered_t *o;
    uint32_t lo, hi, block;
    volatile uint32_t *next;
    pthread_mutex_t *mu;
    uint64_t best;
} mt_arg_t;

static void *mt_worker(void *p)
{
    mt_arg_t *a = (mt_arg_t *)p;
    uint32_t n = a->o->n;
    int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(n + 1));
    a->best = UINT64_MAX;
    if (!buf)
        return NULL;
    for (;;) {
        pthread_mutex_lock(a->mu);
        uint32_t s = *a->next;
        *a->next = s + a->block;
        pthread_mutex_unlock(a->mu);
        if (s >= a->hi)
            break;
        uint32_t e = s + a->block < a->hi ? s + a->block : a->hi;
        uint64_t k = sweep_rows(a->o, s, e, buf, buf + (n + 1),
                                buf + 2 * (n + 1));
        if (k < a->best)
            a->best = k;
    }
    free(buf);
    return NULL;
}

static uint64_t sweep_ordered_mt(const ordered_t *o, uint32_t row_lo, uint32_t row_hi,
                                 int threads);

uint64_t lo_best_move_mt(const float *xy, const uint32_t *route, uint32_t n,
                         uint32_t row_lo, uint32_t row_hi, int threads)
{
    ordered_t o;
    if (ordered_init(&o, xy, route, n)) {
        ordered_free(&o);
        return UINT64_MAX;
    }
    uint64_t best = sweep_ordered_mt(&o, row_lo, row_hi, threads);
    ordered_free(&o);
    return best;
}

/* Rows [row_lo, row_hi) of an ordered tour on `threads` pthreads. */
static uint64_t sweep_ordered_mt(const ordered_t *o, uint32_t row_lo, uint32_t row_hi,
                                 int threads)
{
    const uint32_t n = o->n;
    if (threads < 1)
        threads = 1;
    if (row_lo < 1)
        row_lo = 1;
    if (row_hi == 0 || row_hi > n)
        row_hi = n;
    volatile uint32_t next = row_lo;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    mt_arg_t *args = (mt_arg_t *)malloc(sizeof(mt_arg_t) * threads);
    uint32_t block = 32;
    for (int t = 0; t < threads; t++) {
        args[t].o = o;
        args[t].lo = row_lo;
        args[t].hi = row_hi;
        args[t].block = block;
        args[t].next = &next;
        args[t].mu = &mu;
        args[t].best = UINT64_MAX;
        pthread_create(&th[t], NULL, mt_worker, &args[t]);
    }
    uint64_t best = UINT64_MAX;
    for (int t = 0; t < threads; t++) {
        pthread_join(th[t], NULL);
        if (args[t].best < best)
            best = args[t].best;
    }
    free(th);
    free(args);
    return best;
}

/* ------------------------------------------------------------------------ */
/* Move application, length, descent                                          */
/* ------------------------------------------------------------------------ */

/* rotate(begin, begin+p, end); reverse(begin+(q-p), end) as one gather:
 * new[k] = old[k+p] for k < q-p, else old[(q+n-1-k) mod n]. */
static void rotate_reverse(uint32_t *route, uint32_t n, uint32_t p, uint32_t q,
                           uint32_t *tmp)
{
    uint32_t head = q - p;
    for (uint32_t k = 0; k < n; k++) {
        uint32_t src;
        if (k < head)
            src = k + p;
        else {
            uint64_t s = (uint64_t)q + n - 1 - k;
            src = (uint32_t)(s % n);
        }
        tmp[k] = route[src];
    }
    memcpy(route, tmp, sizeof(uint32_t) * n);
}

/* src/solvers/twoOptLocalSolver.cpp:41-48 */
void lo_apply_move(uint32_t *route, uint32_t n, uint32_t mi, uint32_t mj,
                   uint32_t *tmp)
{
    uint32_t bi = mi, bj = mj;
    if (bj > bi) {
        uint32_t t = bi;
        bi = bj;
        bj = t;
    }
    rotate_reverse(route, n, bj, bi, tmp);
}

/* src/headers.h:170-189.  The reference accumulates the float
 * (sqrtf + 0.5f) values into an unsigned long, which truncates each one; the
 * sum of per-edge nint distances is the same number. */
uint64_t lo_tour_length(const float *xy, const uint32_t *route, uint32_t n)
{
    uint64_t d = 0;
    if (n == 0)
        return 0;
    for (uint32_t i = 1; i < n; i++) {
        const float *a = xy + 2 * (size_t)route[i - 1];
        const float *b = xy + 2 * (size_t)route[i];
        d += (uint64_t)lo_dist(a[0], a[1], b[0], b[1]);
    }
    const float *a = xy + 2 * (size_t)route[n - 1];
    const float *b = xy + 2 * (size_t)route[0];
    d += (uint64_t)lo_dist(a[0], a[1], b[0], b[1]);
    return d;
}

/* src/solvers/twoOptLocalSolver.cpp:22-64; each sweep on `threads` pthreads
 * (the same move: the parallel sweep keeps the lowest-(delta, i, j) rule). */
static void nbr_candidates(const ordered_t *o, const uint32_t *route, const uint32_t *pos,
                           const uint32_t *nbr, uint32_t k, int oropt, int threads,
                           uint64_t *key, uint64_t *or_key);
static uint64_t nbr_sweep(const ordered_t *o, const uint32_t *route, const uint32_t *pos,
                          const uint32_t *nbr, uint32_t k, uint32_t lo, uint32_t hi);
static void or_sweep(const ordered_t *o, const uint32_t *route, const uint32_t *pos,
                     const uint32_t *nbr, uint32_t k, uint32_t lo, uint32_t hi,
                     uint64_t *or_key);
static void apply_oropt(uint32_t *route, uint32_t n, uint32_t s, uint32_t L, uint32_t p,
                        int rev, uint32_t *tmp);

/* With nbr (k cities per city), the neighbour phase of LOGO_SEARCH_NEIGHBOUR
 * comes first: moves from nbr_sweep until none improves, then the full
 * sweeps below; both count towards max_moves (and *nbr_moves gets the
 * first phase's count). */
static int64_t descend_impl(const float *xy, uint32_t *route, uint32_t n,
                            uint64_t max_moves, int32_t *move_log, uint64_t log_cap,
                            int threads, const uint32_t *nbr, uint32_t k,
                            uint64_t *nbr_moves, int oropt)
{
    uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (n + 1));
    int32_t *buf = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(n + 1));
    ordered_t o;
    int64_t moves = 0;
    o.x = (float *)malloc(sizeof(float) * (n + 1));
    o.y = (float *)malloc(sizeof(float) * (n + 1));
    o.e = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
    o.n = n;
    if (nbr_moves)
        *nbr_moves = 0;
    if (nbr && k) {
        uint32_t *pos = (uint32_t *)malloc(sizeof(uint32_t) * (n + 1));
        for (;;) {
            for (uint32_t q = 0; q < n; q++) {
                o.x[q] = xy[2 * (size_t)route[q]];
                o.y[q] = xy[2 * (size_t)route[q] + 1];
                pos[route[q]] = q;
            }
            for (uint32_t q = 1; q < n; q++)
                o.e[q] = lo_dist(o.x[q - 1], o.y[q - 1], o.x[q], o.y[q]);
            o.e[0] = lo_dist(o.x[n - 1], o.y[n - 1], o.x[0], o.y[0]);
            uint64_t key;
            uint64_t ok[5];
            int slot = -1;
            nbr_candidates(&o, route, pos, nbr, k, oropt, threads, &key, ok);
            if (oropt) {
                /* lowest delta; ties to the 2-opt move, then to the lower slot */
                for (int v = 0; v < 5; v++) {
                    if (ok[v] == UINT64_MAX)
                        continue;
                    if (key == UINT64_MAX || (ok[v] >> 42) < (key >> 42)) {
                        key = ok[v];
                        slot = v;
                    }
                }
            }
            if (key == UINT64_MAX)
                break;
            if ((uint64_t)moves >= max_moves) {
                moves = -1;
                break;
            }
            int32_t d;
            uint32_t i, j;
            unpack_key(key, &d, &i, &j);
            if (move_log && (uint64_t)moves < log_cap) {
                move_log[3 * moves + 0] = d;
                move_log[3 * moves + 1] =
                    slot < 0 ? (int32_t)i : -1 - (int32_t)(i + ((uint32_t)slot << 21));
                move_log[3 * moves + 2] = (int32_t)j;
            }
            if (slot < 0)
                lo_apply_move(route, n, i, j, tmp);
            else
                apply_oropt(route, n, i, slot == 0 ? 1u : (uint32_t)((slot + 3) / 2), j,
                            slot == 2 || slot == 4, tmp);
            moves++;
        }
        free(pos);
        if (nbr_moves && moves >= 0)
            *nbr_moves = (uint64_t)moves;
    }
    while (moves >= 0) {
        for (uint32_t k = 0; k < n; k++) {
            o.x[k] = xy[2 * (size_t)route[k]];
            o.y[k] = xy[2 * (size_t)route[k] + 1];
        }
        for (uint32_t k = 1; k < n; k++)
            o.e[k] = lo_dist(o.x[k - 1], o.y[k - 1], o.x[k], o.y[k]);
        uint64_t key = threads > 1 ? sweep_ordered_mt(&o, 1, n, threads)
                                   : sweep_rows(&o, 1, n, buf, buf + (n + 1),
                                                buf + 2 * (n + 1));
        if (key == UINT64_MAX)
            break;
        if ((uint64_t)moves >= max_moves) {
            moves = -1;
            break;
        }
        int32_t d;
        uint32_t i, j;
        unpack_key(key, &d, &i, &j);
        if (move_log && (uint64_t)moves < log_cap) {
            move_log[3 * moves + 0] = d;
            move_log[3 * moves + 1] = (int32_t)i;
            move_log[3 * moves + 2] = (int32_t)j;
        }
        lo_apply_move(route, n, i, j, tmp);
        moves++;
    }
    free(o.x);
    free(o.y);
    free(o.e);
    free(tmp);
    free(buf);
    return moves;
}

int64_t lo_descend(const float *xy, uint32_t *route, uint32_t n,
                   uint64_t max_moves, int32_t *move_log, uint64_t log_cap)
{
    return descend_impl(xy, route, n, max_moves, move_log, log_cap, 1, NULL, 0, NULL, 0);
}

int64_t lo_descend_mt(const float *xy, uint32_t *route, uint32_t n,
                      uint64_t max_moves, int32_t *move_log, uint64_t log_cap,
                      int threads)
{
    return descend_impl(xy, route, n, max_moves, move_log, log_cap, threads, NULL, 0, NULL, 0);
}

/* ------------------------------------------------------------------------ */
/* Neighbour-list search (LOGO_SEARCH_NEIGHBOUR; no reference counterpart)    */
/* ------------------------------------------------------------------------ */

/* k nearest other cities of every city by squared distance in double
 * (dx = (double)x_v - (double)x_u, dx*dx + dy*dy), ties to the lower id,
 * out[v*k + j] nearest first; with fewer than k other cities the remaining
 * slots repeat the last one found (v itself when there is none).  Brute
 * force over all pairs: the test sizes only. */
int lo_knn(const float *xy, uint32_t n, uint32_t k, uint32_t *out)
{
    double *bd = (double *)malloc(sizeof(double) * (k + 1));
    uint32_t *bi = (uint32_t *)malloc(sizeof(uint32_t) * (k + 1));
    if (!bd || !bi) {
        free(bd);
        free(bi);
        return -1;
    }
    for (uint32_t v = 0; v < n; v++) {
        const double px = xy[2 * (size_t)v], py = xy[2 * (size_t)v + 1];
        uint32_t cnt = 0;
        for (uint32_t u = 0; u < n; u++) {
            if (u == v)
                continue;
            const double dx = px - (double)xy[2 * (size_t)u];
            const double dy = py - (double)xy[2 * (size_t)u + 1];
            const double d = dx * dx + dy * dy;
            if (cnt == k && !(d < bd[k - 1] || (d == bd[k - 1] && u < bi[k - 1])))
                continue;
            uint32_t at = cnt < k ? cnt : k - 1;
            while (at > 0 && (d < bd[at - 1] || (d == bd[at - 1] && u < bi[at - 1]))) {
                bd[at] = bd[at - 1];
                bi[at] = bi[at - 1];
                at--;
            }
            bd[at] = d;
            bi[at] = u;
            if (cnt < k)
                cnt++;
        }
        for (uint32_t j = 0; j < k; j++)
            out[(size_t)v * k + j] = cnt == 0 ? v : bi[j < cnt ? j : cnt - 1];
    }
    free(bd);
    free(bi);
    return 0;
}

/* The candidate pairs of one neighbour sweep: for position i (city route[i])
 * and each listed neighbour at position p, (a, b) = (min, max) of (i, p),
 * b >= a + 2: pair (a, b) if a >= 1 and pair (a + 1, b + 1) if
 * b + 1 <= n - 1, i.e. the two full-sweep pairs whose move creates the edge
 * between the two cities.  Lowest improving (delta, i, c) key. */
static uint64_t nbr_sweep(const ordered_t *o, const uint32_t *route, const uint32_t *pos,
                          const uint32_t *nbr, uint32_t k, uint32_t lo, uint32_t hi)
{
    const uint32_t n = o->n;
    const float *X = o->x, *Y = o->y;
    const int32_t *E = o->e;
    uint64_t best = UINT64_MAX;
    for (uint32_t i = lo; i < hi && i < n; i++) {
        const uint32_t t = route[i];
        for (uint32_t q = 0; q < k; q++) {
            const uint32_t p = pos[nbr[(size_t)t * k + q]];
            const uint32_t a = i < p ? i : p, b = i < p ? p : i;
            if (b < a + 2)
                continue;
            const int32_t D = lo_dist(X[a], Y[a], X[b], Y[b]);
            if (a >= 1) {
                const int32_t delta = D + lo_dist(X[a - 1], Y[a - 1], X[b - 1], Y[b - 1]) -
                                      E[a] - E[b];
                if (delta < 0) {
                    const uint64_t key = lo_pack_key(delta, a, b);
                    if (key < best)
                        best = key;
                }
            }
            if (b + 1 <= n - 1) {
                const int32_t delta = lo_dist(X[a + 1], Y[a + 1], X[b + 1], Y[b + 1]) + D -
                                      E[a + 1] - E[b + 1];
                if (delta < 0) {
                    const uint64_t key = lo_pack_key(delta, a + 1, b + 1);
                    if (key < best)
                        best = key;
                }
            }
        }
    }
    return best;
}

typedef struct {
    const ordered_t *o;
    const uint32_t *route, *pos, *nbr;
    uint32_t k, lo, hi;
    int oropt;
    uint64_t key, or_key[5];
} nbr_job_t;

static void *nbr_worker(void *p)
{
    nbr_job_t *j = (nbr_job_t *)p;
    j->key = nbr_sweep(j->o, j->route, j->pos, j->nbr, j->k, j->lo, j->hi);
    for (int v = 0; v < 5; v++)
        j->or_key[v] = UINT64_MAX;
    if (j->oropt)
        or_sweep(j->o, j->route, j->pos, j->nbr, j->k, j->lo, j->hi, j->or_key);
    return NULL;
}

/* The neighbour sweep's lowest 2-opt key and Or-opt slot keys, positions
 * split over `threads` pthreads (the minima do not depend on the split). */
static void nbr_candidates(const ordered_t *o, const uint32_t *route, const uint32_t *pos,
                           const uint32_t *nbr, uint32_t k, int oropt, int threads,
                           uint64_t *key, uint64_t *or_key)
{
    const uint32_t n = o->n;
    if (threads < 1)
        threads = 1;
    if (threads > 64)
        threads = 64;
    if ((uint32_t)threads > n / 256 + 1)
        threads = (int)(n / 256 + 1);
    nbr_job_t jobs[64];
    pthread_t tid[64];
    int started[64];
    for (int t = 0; t < threads; t++) {
        jobs[t].o = o;
        jobs[t].route = route;
        jobs[t].pos = pos;
        jobs[t].nbr = nbr;
        jobs[t].k = k;
        jobs[t].oropt = oropt;
        jobs[t].lo = (uint32_t)((uint64_t)n * t / threads);
        jobs[t].hi = (uint32_t)((uint64_t)n * (t + 1) / threads);
        started[t] = t > 0 && pthread_create(&tid[t], NULL, nbr_worker, &jobs[t]) == 0;
    }
    nbr_worker(&jobs[0]);
    for (int t = 1; t < threads; t++) {
        if (started[t])
            pthread_join(tid[t], NULL);
        else
            nbr_worker(&jobs[t]);
    }
    *key = UINT64_MAX;
    for (int v = 0; v < 5; v++)
        or_key[v] = UINT64_MAX;
    for (int t = 0; t < threads; t++) {
        if (jobs[t].key < *key)
            *key = jobs[t].key;
        for (int v = 0; v < 5; v++)
            if (jobs[t].or_key[v] < or_key[v])
                or_key[v] = jobs[t].or_key[v];
    }
}

int64_t lo_descend_nbr(const float *xy, uint32_t *route, uint32_t n, const uint32_t *nbr,
                       uint32_t k, uint64_t max_moves, int threads, uint64_t *nbr_moves,
                       int oropt)
{
    return descend_impl(xy, route, n, max_moves, NULL, 0, threads, nbr, k, nbr_moves, oropt);
}

/* One step of the neighbour search on `route` without applying it: the
 * chosen move's delta, slot (-1 for 2-opt, else the Or-opt variant) and
 * (i, j) = (first, second field of its key); returns 0, or 1 when no
 * candidate improves. */
int lo_nbr_step(const float *xy, const uint32_t *route, uint32_t n, const uint32_t *nbr,
                uint32_t k, int oropt, int32_t *delta, int32_t *slot, uint32_t *i, uint32_t *j)
{
    ordered_t o;
    uint32_t *pos = (uint32_t *)malloc(sizeof(uint32_t) * (n + 1));
    if (!pos || ordered_init(&o, xy, route, n)) {
        free(pos);
        return -1;
    }
    for (uint32_t q = 0; q < n; q++)
        pos[route[q]] = q;
    uint64_t key;
    uint64_t ok[5];
    int sl = -1;
    nbr_candidates(&o, route, pos, nbr, k, oropt, 1, &key, ok);
    if (oropt) {
        for (int v = 0; v < 5; v++) {
            if (ok[v] == UINT64_MAX)
                continue;
            if (key == UINT64_MAX || (ok[v] >> 42) < (key >> 42)) {
                key = ok[v];
                sl = v;
            }
        }
    }
    ordered_free(&o);
    free(pos);
    if (key == UINT64_MAX)
        return 1;
    unpack_key(key, delta, i, j);
    *slot = sl;
    return 0;
}

/* Or-opt moves (LOGO_SEARCH_NEIGHBOUR_OROPT): segment [s, s+L), L = 1..3,
 * 1 <= s, s+L <= n-1, moved into the gap after old position p (p <= s-2, or
 * s+L <= p <= n-2), in order or reversed.  Candidates are the moves that
 * create an edge from a segment end to one of its listed neighbours (the
 * city at s starts every segment; the city at s+L-1 ends the one of length
 * L).  Slot v = (L1, L2, L2 reversed, L3, L3 reversed) keeps the lowest
 * improving pack_key(delta, s, p). */
static void or_try(const ordered_t *o, uint32_t s, uint32_t L, int rev, uint32_t p,
                   int32_t base, int have, uint64_t *or_key)
{
    const uint32_t n = o->n;
    if (!have)
        return;
    if (!(p + 2 <= s || (p >= s + L && p + 2 <= n)))
        return;
    const uint32_t u = rev ? s + L - 1 : s, w = rev ? s : s + L - 1;
    /* both new distances are >= 0: the first alone may already rule it out */
    const int32_t part = base + lo_dist(o->x[p], o->y[p], o->x[u], o->y[u]) - o->e[p + 1];
    if (part >= 0)
        return;
    const int32_t delta = part + lo_dist(o->x[w], o->y[w], o->x[p + 1], o->y[p + 1]);
    if (delta < 0) {
        const int v = L == 1 ? 0 : (int)(2 * L - 3) + (rev ? 1 : 0);
        const uint64_t key = lo_pack_key(delta, s, p);
        if (key < or_key[v])
            or_key[v] = key;
    }
}

static void or_sweep(const ordered_t *o, const uint32_t *route, const uint32_t *pos,
                     const uint32_t *nbr, uint32_t k, uint32_t lo, uint32_t hi,
                     uint64_t *or_key)
{
    const uint32_t n = o->n;
    for (uint32_t s = lo < 1 ? 1 : lo; s < hi && s + 2 <= n; s++) {
        int32_t base[3];
        int have[3];
        for (uint32_t L = 1; L <= 3; L++) {
            have[L - 1] = s + L <= n - 1;
            base[L - 1] = have[L - 1] ? lo_dist(o->x[s - 1], o->y[s - 1], o->x[s + L],
                                                o->y[s + L]) - o->e[s] - o->e[s + L]
                                      : 0;
        }
        for (uint32_t anchor = 0; anchor < 3; anchor++) {
            if (anchor >= 1 && !have[anchor])
                break;
            const uint32_t c = route[s + anchor];
            for (uint32_t t = 0; t < k; t++) {
                const uint32_t q = pos[nbr[(size_t)c * k + t]];
                if (anchor == 0) {
                    or_try(o, s, 1, 0, q, base[0], have[0], or_key);
                    if (q >= 1)
                        or_try(o, s, 1, 0, q - 1, base[0], have[0], or_key);
                    for (uint32_t L = 2; L <= 3; L++) {
                        or_try(o, s, L, 0, q, base[L - 1], have[L - 1], or_key);
                        if (q >= 1)
                            or_try(o, s, L, 1, q - 1, base[L - 1], have[L - 1], or_key);
                    }
                } else {
                    const uint32_t L = anchor + 1;
                    if (q >= 1)
                        or_try(o, s, L, 0, q - 1, base[L - 1], have[L - 1], or_key);
                    or_try(o, s, L, 1, q, base[L - 1], have[L - 1], or_key);
                }
            }
        }
    }
}

/* The segment moves right: old[0,s) old[s+L,p] seg old[p+1,n); left:
 * old[0,p] seg old[p+1,s) old[s+L,n); seg reversed when rev. */
static void apply_oropt(uint32_t *route, uint32_t n, uint32_t s, uint32_t L, uint32_t p,
                        int rev, uint32_t *tmp)
{
    uint32_t q = 0;
    if (p >= s + L) {
        for (uint32_t t = 0; t < s; t++) tmp[q++] = route[t];
        for (uint32_t t = s + L; t <= p; t++) tmp[q++] = route[t];
        for (uint32_t t = 0; t < L; t++) tmp[q++] = route[rev ? s + L - 1 - t : s + t];
        for (uint32_t t = p + 1; t < n; t++) tmp[q++] = route[t];
    } else {
        for (uint32_t t = 0; t <= p; t++) tmp[q++] = route[t];
        for (uint32_t t = 0; t < L; t++) tmp[q++] = route[rev ? s + L - 1 - t : s + t];
        for (uint32_t t = p + 1; t < s; t++) tmp[q++] = route[t];
        for (uint32_t t = s + L; t < n; t++) tmp[q++] = route[t];
    }
    memcpy(route, tmp, sizeof(uint32_t) * n);
}

/* ------------------------------------------------------------------------ */
/* Kicks and ILS                                                              */
/* ------------------------------------------------------------------------ */

/* src/solvers/ILSGlobalSolver.cpp:37-48 */
void lo_kick_segment(uint32_t *route, uint32_t n, uint64_t *rng, uint32_t *tmp)
{
    uint32_t a = lo_uniform(rng, n);
    uint32_t b = lo_uniform(rng, n);
    if (b < a) {
        uint32_t t = a;
        a = b;
        b = t;
    }
    rotate_reverse(route, n, a, b, tmp);
}

void lo_kick_double_bridge(uint32_t *route, uint32_t n, uint64_t *rng,
                           uint32_t *tmp)
{
    if (n < 2)
        return;
    uint32_t p[3];
    for (int k = 0; k < 3; k++)
        p[k] = 1 + lo_uniform(rng, n - 1);
    /* sort three */
    if (p[1] < p[0]) { uint32_t t = p[0]; p[0] = p[1]; p[1] = t; }
    if (p[2] < p[1]) { uint32_t t = p[1]; p[1] = p[2]; p[2] = t; }
    if (p[1] < p[0]) { uint32_t t = p[0]; p[0] = p[1]; p[1] = t; }
    uint32_t k = 0;
    for (uint32_t s = 0; s < p[0]; s++) tmp[k++] = route[s];
    for (uint32_t s = p[1]; s < p[2]; s++) tmp[k++] = route[s];
    for (uint32_t s = p[0]; s < p[1]; s++) tmp[k++] = route[s];
    for (uint32_t s = p[2]; s < n; s++) tmp[k++] = route[s];
    memcpy(route, tmp, sizeof(uint32_t) * n);
}

/* src/solvers/ILSGlobalSolverSequential.cpp:60-100, stop rule replaced by an
 * explicit kick count (the reference's stop test needs a known optimum,
 * :98-99, and ends after one pass otherwise). */
static int ils_impl(const float *xy, uint32_t *route, uint32_t n, uint32_t kicks,
                    uint64_t seed, int kick_kind, uint64_t max_moves_per_descent,
                    lo_ils_stats *stats, int threads, const uint32_t *nbr, uint32_t k,
                    int oropt)
{
    uint32_t *best = (uint32_t *)malloc(sizeof(uint32_t) * (n + 1));
    uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (n + 1));
    uint64_t rng = seed;
    lo_ils_stats st;
    int rc = 0;
    memset(&st, 0, sizeof(st));
    st.start_length = lo_tour_length(xy, route, n);
    uint64_t best_len = st.start_length;
    memcpy(best, route, sizeof(uint32_t) * n);
    for (uint32_t it = 0;; it++) {
        int64_t m = descend_impl(xy, route, n, max_moves_per_descent, NULL, 0, threads, nbr, k,
                                 NULL, oropt);
        st.descents++;
        if (m < 0) {
            rc = -1;
            break;
        }
        st.moves += (uint64_t)m;
        uint64_t len = lo_tour_length(xy, route, n);
        if (len < best_len) {
            best_len = len;
            memcpy(best, route, sizeof(uint32_t) * n);
            st.accepted++;
        } else {
            memcpy(route, best, sizeof(uint32_t) * n);
        }
        if (it == kicks)
            break;
        if (kick_kind == LO_KICK_DOUBLE_BRIDGE)
            lo_kick_double_bridge(route, n, &rng, tmp);
        else
            lo_kick_segment(route, n, &rng, tmp);
    }
    memcpy(route, best, sizeof(uint32_t) * n);
    st.best_length = best_len;
    if (stats)
        *stats = st;
    free(best);
    free(tmp);
    return rc;
}

int lo_ils(const float *xy, uint32_t *route, uint32_t n, uint32_t kicks,
           uint64_t seed, int kick_kind, uint64_t max_moves_per_descent,
           lo_ils_stats *stats)
{
    return ils_impl(xy, route, n, kicks, seed, kick_kind, max_moves_per_descent, stats, 1,
                    NULL, 0, 0);
}

int lo_ils_mt(const float *xy, uint32_t *route, uint32_t n, uint32_t kicks,
              uint64_t seed, int kick_kind, uint64_t max_moves_per_descent,
              lo_ils_stats *stats, int threads)
{
    return ils_impl(xy, route, n, kicks, seed, kick_kind, max_moves_per_descent, stats,
                    threads, NULL, 0, 0);
}

int lo_ils_nbr(const float *xy, uint32_t *route, uint32_t n, uint32_t kicks, uint64_t seed,
               int kick_kind, uint64_t max_moves_per_descent, lo_ils_stats *stats,
               int threads, const uint32_t *nbr, uint32_t k, int oropt)
{
    return ils_impl(xy, route, n, kicks, seed, kick_kind, max_moves_per_descent, stats,
                    threads, nbr, k, oropt);
}

/* ------------------------------------------------------------------------ */
/* Nearest-neighbour start tour                                               */
/* ------------------------------------------------------------------------ */

/* initRoute_KD_NN (src/utils/kdtree_utils.c:279-301) searches a kd-tree over
 * double coordinates with Euclidean distance sqrt(dx*dx + dy*dy) in double
 * (src/kdtree++/function.hpp:34-45, node.hpp:195-345).  This restatement
 * uses a uniform bucket grid and the same distance; where two candidates are
 * exactly as near, the lower city id wins (the reference's choice there
 * depends on tree traversal order), and the tie is counted. */
typedef struct {
    uint32_t *start, *count, *items;
    double x0, y0, inv;
    uint32_t gw, gh;
} grid_t;

static double nn_d(const float *xy, uint32_t a, double px, double py)
{
    double dx = px - (double)xy[2 * (size_t)a];
    double dy = py - (double)xy[2 * (size_t)a + 1];
    return sqrt(dx * dx + dy * dy);
}

uint64_t lo_nn_tour(const float *xy, uint32_t n, uint32_t *route)
{
    uint64_t ties = 0;
    if (n == 0)
        return 0;
    double x0 = xy[0], y0 = xy[1], x1 = xy[0], y1 = xy[1];
    for (uint32_t k = 1; k < n; k++) {
        double x = xy[2 * (size_t)k], y = xy[2 * (size_t)k + 1];
        if (x < x0) x0 = x;
        if (x > x1) x1 = x;
        if (y < y0) y0 = y;
        if (y > y1) y1 = y;
    }
    double w = x1 - x0, h = y1 - y0;
    if (w <= 0) w = 1;
    if (h <= 0) h = 1;
    double cell = sqrt(w * h / ((double)n / 2.0 + 1.0));
    if (cell <= 0) cell = 1;
    grid_t g;
    g.gw = (uint32_t)(w / cell) + 1;
    g.gh = (uint32_t)(h / cell) + 1;
    if (g.gw > 4096) g.gw = 4096;
    if (g.gh > 4096) g.gh = 4096;
    g.x0 = x0;
    g.y0 = y0;
    double cw = w / g.gw, ch = h / g.gh;
    if (cw <= 0) cw = 1;
    if (ch <= 0) ch = 1;
    size_t ncell = (size_t)g.gw * g.gh;
    g.start = (uint32_t *)calloc(ncell + 1, sizeof(uint32_t));
    g.count = (uint32_t *)calloc(ncell, sizeof(uint32_t));
    g.items = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint32_t *cellof = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint32_t *pos = (uint32_t *)malloc(sizeof(uint32_t) * n);
    for (uint32_t k = 0; k < n; k++) {
        uint32_t cx = (uint32_t)(((double)xy[2 * (size_t)k] - x0) / cw);
        uint32_t cy = (uint32_t)(((double)xy[2 * (size_t)k + 1] - y0) / ch);
        if (cx >= g.gw) cx = g.gw - 1;
        if (cy >= g.gh) cy = g.gh - 1;
        cellof[k] = cy * g.gw + cx;
        g.count[cellof[k]]++;
    }
    for (size_t c = 0; c < ncell; c++)
        g.start[c + 1] = g.start[c] + g.count[c];
    memset(g.count, 0, sizeof(uint32_t) * ncell);
    for (uint32_t k = 0; k < n; k++) {
        uint32_t c = cellof[k];
        pos[k] = g.start[c] + g.count[c];
        g.items[pos[k]] = k;
        g.count[c]++;
    }
    /* live items of cell c: items[start[c] .. start[c]+count[c]) */
    uint32_t cur = 0;
    double px = xy[0], py = xy[1];
    for (uint32_t step = 0; step < n; step++) {
        /* search rings outward until the ring's minimum possible distance
         * exceeds the best found */
        uint32_t pcx = (uint32_t)((px - x0) / cw);
        uint32_t pcy = (uint32_t)((py - y0) / ch);
        if (pcx >= g.gw) pcx = g.gw - 1;
        if (pcy >= g.gh) pcy = g.gh - 1;
        double bestd = INFINITY;
        uint32_t besti = UINT32_MAX;
        uint32_t maxr = g.gw > g.gh ? g.gw : g.gh;
        for (uint32_t r = 0; r <= maxr; r++) {
            if (besti != UINT32_MAX) {
                double ring = ((double)r - 1.0) * (cw < ch ? cw : ch);
                if (ring > bestd)
                    break;
            }
            int64_t xa = (int64_t)pcx - r, xb = (int64_t)pcx + r;
            int64_t ya = (int64_t)pcy - r, yb = (int64_t)pcy + r;
            for (int64_t cy = ya; cy <= yb; cy++) {
                if (cy < 0 || cy >= (int64_t)g.gh)
                    continue;
                int edge_row = (cy == ya || cy == yb);
                for (int64_t cx = xa; cx <= xb; cx++) {
                    if (cx < 0 || cx >= (int64_t)g.gw)
                        continue;
                    if (!edge_row && cx != xa && cx != xb)
                        continue;
                    size_t c = (size_t)cy * g.gw + (size_t)cx;
                    for (uint32_t t = 0; t < g.count[c]; t++) {
                        uint32_t id = g.items[g.start[c] + t];
                        double d = nn_d(xy, id, px, py);
                        if (d < bestd) {
                            bestd = d;
                            besti = id;
                        } else if (d == bestd) {
                            ties++;
                            if (id < besti)
                                besti = id;
                        }
                    }
                }
            }
        }
        /* the first pick is city 0 itself (distance 0), as in the
         * reference where the search starts at city 0's own point */
        if (step == 0)
            besti = besti == UINT32_MAX ? 0 : besti;
        route[step] = besti;
        /* remove besti: swap with the last live item of its cell */
        uint32_t c = cellof[besti];
        uint32_t last = g.start[c] + g.count[c] - 1;
        uint32_t moved = g.items[last];
        g.items[pos[besti]] = moved;
        pos[moved] = pos[besti];
        g.items[last] = besti;
        pos[besti] = last;
        g.count[c]--;
        cur = besti;
        px = xy[2 * (size_t)cur];
        py = xy[2 * (size_t)cur + 1];
    }
    free(g.start);
    free(g.count);
    free(g.items);
    free(cellof);
    free(pos);
    return ties;
}

/* src/utils/construction.c:152-183 */
int lo_check_tour(const uint32_t *route, uint32_t n)
{
    uint8_t *seen = (uint8_t *)calloc(n ? n : 1, 1);
    int ok = 1;
    for (uint32_t k = 0; k < n && ok; k++) {
        if (route[k] >= n || seen[route[k]])
            ok = 0;
        else
            seen[route[k]] = 1;
    }
    free(seen);
    return ok;
}

/* ------------------------------------------------------------------------ */
/* Batch of ILS runs on host threads                                          */
/* ------------------------------------------------------------------------ */

typedef struct {
    const float *xy;
    uint32_t *routes;
    const uint64_t *offsets;
    const uint32_t *ns;
    const uint64_t *seeds;
    uint32_t count, kicks;
    int kind;
    volatile uint32_t *next;
    pthread_mutex_t *mu;
    uint64_t *lens, *moves;
    int rc;
} batch_arg_t;

static void *batch_worker(void *p)
{
    batch_arg_t *a = (batch_arg_t *)p;
    for (;;) {
        pthread_mutex_lock(a->mu);
        uint32_t k = *a->next;
        *a->next = k + 1;
        pthread_mutex_unlock(a->mu);
        if (k >= a->count)
            break;
        lo_ils_stats st;
        uint64_t off = a->offsets[k];
        uint32_t n = a->ns[k];
        int rc = lo_ils(a->xy + 2 * off, a->routes + off, n, a->kicks,
                        a->seeds[k], a->kind, (uint64_t)64 * n * n + 1024, &st);
        if (rc)
            a->rc = rc;
        a->lens[k] = st.best_length;
        if (a->moves)
            a->moves[k] = st.moves;
    }
    return NULL;
}

int lo_ils_batch(const float *xy, uint32_t *routes, const uint64_t *offsets,
                 const uint32_t *ns, const uint64_t *seeds, uint32_t count,
                 uint32_t kicks, int kick_kind, int threads,
                 uint64_t *best_lengths, uint64_t *moves)
{
    if (threads < 1)
        threads = 1;
    volatile uint32_t next = 0;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    batch_arg_t *args = (batch_arg_t *)malloc(sizeof(batch_arg_t) * threads);
    for (int t = 0; t < threads; t++) {
        batch_arg_t *a = &args[t];
        a->xy = xy;
        a->routes = routes;
        a->offsets = offsets;
        a->ns = ns;
        a->seeds = seeds;
        a->count = count;
        a->kicks = kicks;
        a->kind = kick_kind;
        a->next = &next;
        a->mu = &mu;
        a->lens = best_lengths;
        a->moves = moves;
        a->rc = 0;
        pthread_create(&th[t], NULL, batch_worker, a);
    }
    int rc = 0;
    for (int t = 0; t < threads; t++) {
        pthread_join(th[t], NULL);
        if (args[t].rc)
            rc = args[t].rc;
    }
    free(th);
    free(args);
    return rc;
}
