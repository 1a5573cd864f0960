// GPUSolver: the reference-side binding of the GB300 engine, as a maintainer
// adds it to the LOGO TSP solver tree (src/solvers/GPUSolver.h there).
//
// A TwoOptLocalSolver (src/solvers/twoOptLocalSolver.h:23-70) whose
// LocalSolver methods (src/solvers/localSolver.h:116-125) forward to the C ABI
// of include/logo_gpu.h: init/close create and destroy a context,
// optimizeStep is one device sweep (logo_best_move), optimize the whole
// descent on the device (logo_descend: one call instead of one
// H2D/launch/D2H round trip per move, CUDASolver.cpp:285-386), benchmark times
// one step.  city_coords / logo_xy (src/defs.h:173-178) and best2_out /
// logo_move (src/defs.h:181-187) have the same layout.  Errors follow the
// reference's own policy for its CUDA backend: message and exit(-1)
// (src/utils/UtilsCUDA.cpp:318-328).
//
// Compiled against the reference headers and linked against liblogo_gpu.so by
// tests/test_integration_build.py.
#ifndef LOGO_GB300_GPU_SOLVER_H
#define LOGO_GB300_GPU_SOLVER_H

#include <sys/time.h>

#include <cstdio>
#include <cstdlib>

#include <twoOptLocalSolver.h>

#include "logo_gpu.h"

static_assert(sizeof(city_coords) == sizeof(logo_xy), "city_coords and logo_xy differ");
static_assert(sizeof(best2_out) == sizeof(logo_move), "best2_out and logo_move differ");

class GPUSolver : public TwoOptLocalSolver {
public:
    GPUSolver(city_coords *c, cmdArguments *a, string d, short dev, ROUTE_DATA_TYPE n)
        : TwoOptLocalSolver(c, a, d, dev, n) {
        init();
    }
    ~GPUSolver() { close(); }

    void init() {
        if (ctx) return;
        if (logo_ctx_create((int)deviceId, (const logo_xy *)coords, (uint32_t)size, &ctx) !=
            LOGO_OK) {
            fprintf(stderr, "GPUSolver: %s\n", logo_last_error(NULL));
            exit(-1);
        }
    }

    void close() {
        if (ctx) logo_ctx_destroy(ctx);
        ctx = NULL;
    }

    // TwoOptLocalSolver::optimize (twoOptLocalSolver.cpp:22-64) on the device:
    // the route is overwritten with the local optimum.
    void optimize(vector<ROUTE_DATA_TYPE> &route, vector<unsigned long> &bestLength) {
        (void)bestLength;
        logo_stats st;
        if (logo_descend(ctx, route.data(), 0, &st) != LOGO_OK) {
            fprintf(stderr, "GPUSolver: %s\n", logo_last_error(ctx));
            exit(-1);
        }
    }

    struct process_time benchmark(vector<ROUTE_DATA_TYPE> &route) {
        struct process_time t;
        struct timeval s, e;
        gettimeofday(&s, NULL);
        t.out = optimizeStep(route);
        gettimeofday(&e, NULL);
        t.kernel_time = (double)(e.tv_sec - s.tv_sec) + 1e-6 * (double)(e.tv_usec - s.tv_usec);
        t.HtD_time = t.DtH_time = 0;
        return t;
    }

    // ILSGlobalSolverSequential::optimize (ILSGlobalSolverSequential.cpp:60-100)
    // with a kick count instead of the known-optimum stop, all on the device.
    void ils(vector<ROUTE_DATA_TYPE> &route, uint32_t kicks, uint64_t seed) {
        logo_stats st;
        if (logo_ils(ctx, route.data(), kicks, seed, LOGO_KICK_SEGMENT, &st) != LOGO_OK) {
            fprintf(stderr, "GPUSolver: %s\n", logo_last_error(ctx));
            exit(-1);
        }
    }

protected:
    struct best2_out optimizeStep(const vector<ROUTE_DATA_TYPE> &route) {
        logo_move m;
        if (logo_best_move(ctx, route.data(), &m) != LOGO_OK) {
            fprintf(stderr, "GPUSolver: %s\n", logo_last_error(ctx));
            exit(-1);
        }
        struct best2_out o;
        o.i = m.i;
        o.j = m.j;
        o.minchange = m.minchange;
        return o;
    }

private:
    logo_ctx *ctx = NULL;
};

#endif
