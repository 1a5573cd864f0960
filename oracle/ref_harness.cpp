// Harness that runs the reference's own C++ code for the 2-opt path, used to
// pin the oracle (TEST INFRASTRUCTURE ONLY).  It is compiled together with the
// unmodified reference sources by oracle/build_ref.sh into oracle/_ref/ and
// is never shipped or linked into the product.
//
// What runs from the reference here:
//   TwoOptLocalSolver::optimize      src/solvers/twoOptLocalSolver.cpp:22-64
//   routeLength                      src/headers.h:170-189
//   ILSGlobalSolver::kick            src/solvers/ILSGlobalSolver.cpp:37-48
//   ILSGlobalSolverSequential::optimize
//                                    src/solvers/ILSGlobalSolverSequential.cpp:60-100
//   CPUSolver::optimizeStep (AVX)    src/solvers/cpuSolver.cpp:143-230
//   constructKDTree/initRoute_KD_NN  src/utils/kdtree_utils.c:29-52,279-301
//   multipleFragment_KD              src/utils/kdtree_utils.c:56-242
//   readFileCoords                   src/utils/tsp_loader.c:49-162
// What this file adds: NintCPUSolver, whose optimizeStep is the loop of
// CPUSolver::optimizeStep (i ascending, j ascending, strict <, report
// (i, j+1)) with the per-edge nint distance of src/cuda/cuda_common.h:33-40,
// and a rand() replacement (SplitMix64) so kicks follow a seed.
//
// Usage: ref_harness <cmd> <in> <out> [args]   (binary files, see main()).
#include <cpuSolver.h>
#include <ILSGlobalSolverSequential.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

// ---- seeded rand() replacement ------------------------------------------
static uint64_t g_rng = 0;
static uint32_t g_rng_n = 1;
static uint64_t g_rand_calls = 0;
static uint64_t g_stop_after_calls = UINT64_MAX;
static void (*g_on_stop)(void) = nullptr;

static uint64_t splitmix64(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ILSGlobalSolver.cpp is compiled with ref_rand_hook.h force-included, so its
// rand() is logo_ref_rand: each draw is
// uniform in [0, g_rng_n), so the kick's `rand() % route.size()` keeps it.
extern "C" int logo_ref_rand(void) {
    uint64_t hi = splitmix64(&g_rng) >> 32;
    g_rand_calls++;
    if (g_rand_calls == g_stop_after_calls && g_on_stop) g_on_stop();
    return (int)((hi * (uint64_t)g_rng_n) >> 32);
}

// ---- per-edge nint local solver --------------------------------------------
static std::vector<int32_t> g_log;

class NintCPUSolver : public TwoOptLocalSolver {
public:
    NintCPUSolver(city_coords *c, cmdArguments *a, ROUTE_DATA_TYPE n)
        : TwoOptLocalSolver(c, a, "nint", 0, n) {}
    void init() {}
    void close() {}
    struct process_time benchmark(vector<ROUTE_DATA_TYPE> &route) {
        struct process_time t;
        t.out = optimizeStep(route);
        t.kernel_time = t.HtD_time = t.DtH_time = 0;
        return t;
    }
    uint64_t steps = 0;

protected:
    struct best2_out optimizeStep(const vector<ROUTE_DATA_TYPE> &route) {
        struct best2_out out;
        out.minchange = 0;
        out.i = 0;
        out.j = 0;
        steps++;
        const ROUTE_DATA_TYPE n = route.size();
        std::vector<float> X(n), Y(n);
        for (ROUTE_DATA_TYPE k = 0; k < n; k++) {
            X[k] = coords[route[k]].x;
            Y[k] = coords[route[k]].y;
        }
        for (ROUTE_DATA_TYPE i = 1; i < n - 2; i++) {
            int const1 = (int)calculateDistance2D(i, i - 1, X.data(), Y.data());
            for (ROUTE_DATA_TYPE j = i + 1; j < n - 1; j++) {
                int change = (int)calculateDistance2D(i, j + 1, X.data(), Y.data()) +
                             (int)calculateDistance2D(i - 1, j, X.data(), Y.data()) -
                             const1 -
                             (int)calculateDistance2D(j + 1, j, X.data(), Y.data());
                if (change < 0 && change < out.minchange) {
                    out.minchange = change;
                    out.i = i;
                    out.j = j + 1;
                }
            }
        }
        if (out.minchange < 0) {
            g_log.push_back(out.minchange);
            g_log.push_back((int32_t)out.i);
            g_log.push_back((int32_t)out.j);
        }
        return out;
    }
};

class AvxProbe : public CPUSolver {
public:
    AvxProbe(city_coords *c, cmdArguments *a, ROUTE_DATA_TYPE n)
        : CPUSolver(c, a, "avx", 0, n) {}
    struct best2_out step(const vector<ROUTE_DATA_TYPE> &r) { return optimizeStep(r); }
};

class IlsProbe;
static IlsProbe *g_probe = nullptr;

class IlsProbe : public ILSGlobalSolverSequential {
public:
    IlsProbe(city_coords *c, cmdArguments *a, ROUTE_DATA_TYPE n)
        : ILSGlobalSolverSequential(c, a, "ref", TYPE_GLOBAL_SOLVER_CPU, n) {
        delete localSolver;  // replace the AVX CPUSolver made by init()
        localSolver = new NintCPUSolver(c, a, n);
        solution = 0;  // keeps the reference's stop test true until stop()
        timelimit = 0;
    }
    void kickOnce(vector<ROUTE_DATA_TYPE> &r) { kick(r); }
    void stop() { solution = (unsigned long)1 << 62; }
    static vector<ROUTE_DATA_TYPE> best() { return bestGlobalMinima.back(); }
    static unsigned long bestLength() { return bestGlobalMinimaLengths.back(); }
};

static void stop_probe(void) {
    if (g_probe) g_probe->stop();
}

// ---- I/O ---------------------------------------------------------------------
// input file: u32 n, float xy[2n], u32 route[n]
static bool read_input(const char *path, std::vector<city_coords> &c,
                       std::vector<ROUTE_DATA_TYPE> &r) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    uint32_t n = 0;
    bool ok = fread(&n, 4, 1, f) == 1;
    c.resize(n);
    r.resize(n);
    for (uint32_t k = 0; ok && k < n; k++)
        ok = fread(&c[k].x, 4, 1, f) == 1 && fread(&c[k].y, 4, 1, f) == 1;
    if (ok && n) ok = fread(r.data(), 4, n, f) == n;
    fclose(f);
    return ok;
}

static void put_u64(FILE *f, uint64_t v) { fwrite(&v, 8, 1, f); }
static void put_route(FILE *f, const std::vector<ROUTE_DATA_TYPE> &r) {
    uint32_t n = r.size();
    fwrite(&n, 4, 1, f);
    if (n) fwrite(r.data(), 4, n, f);
}

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: ref_harness cmd in out [args]\n");
        return 2;
    }
    std::string cmd = argv[1];
    static char outname[] = "/dev/null";
    cmdArguments args;
    memset(&args, 0, sizeof(args));
    args.outfilename = outname;
    args.showLocalOptimizationInfo = 0;
    args.solution = 1;
    std::vector<city_coords> c;
    std::vector<ROUTE_DATA_TYPE> r;
    FILE *out = nullptr;

    if (cmd == "tsp") {  // readFileCoords on a TSPLIB file
        std::vector<city_coords> buf(MAX_CITIES);
        int n = readFileCoords(argv[2], buf.data());
        out = fopen(argv[3], "wb");
        uint32_t un = n;
        fwrite(&un, 4, 1, out);
        for (int k = 0; k < n; k++) {
            fwrite(&buf[k].x, 4, 1, out);
            fwrite(&buf[k].y, 4, 1, out);
        }
        fclose(out);
        return 0;
    }
    if (!read_input(argv[2], c, r)) {
        fprintf(stderr, "bad input\n");
        return 2;
    }
    const ROUTE_DATA_TYPE n = r.size();
    out = fopen(argv[3], "wb");
    if (!out) return 2;

    if (cmd == "descend") {  // TwoOptLocalSolver::optimize with nint steps
        NintCPUSolver s(c.data(), &args, n);
        std::vector<unsigned long> best;
        best.push_back(routeLength(r, c.data()));
        s.optimize(r, best);
        put_u64(out, g_log.size() / 3);
        if (!g_log.empty()) fwrite(g_log.data(), 4, g_log.size(), out);
        put_route(out, r);
        put_u64(out, routeLength(r, c.data()));
    } else if (cmd == "step") {  // one nint optimizeStep
        NintCPUSolver s(c.data(), &args, n);
        struct process_time t = s.benchmark(r);
        int32_t v[3] = {t.out.minchange, (int32_t)t.out.i, (int32_t)t.out.j};
        fwrite(v, 4, 3, out);
    } else if (cmd == "avxstep") {  // CPUSolver::optimizeStep as shipped (AVX)
        AvxProbe s(c.data(), &args, n);
        struct best2_out o = s.step(r);
        int32_t v[3] = {o.minchange, (int32_t)o.i, (int32_t)o.j};
        fwrite(v, 4, 3, out);
    } else if (cmd == "length") {
        put_u64(out, routeLength(r, c.data()));
    } else if (cmd == "kick") {  // ILSGlobalSolver::kick, `count` times
        if (argc < 6) return 2;
        g_rng = strtoull(argv[4], nullptr, 0);
        g_rng_n = n;
        uint64_t count = strtoull(argv[5], nullptr, 0);
        IlsProbe p(c.data(), &args, n);
        for (uint64_t k = 0; k < count; k++) p.kickOnce(r);
        put_route(out, r);
        put_u64(out, g_rng);
    } else if (cmd == "ils") {  // ILSGlobalSolverSequential::optimize
        if (argc < 6) return 2;
        uint64_t kicks = strtoull(argv[4], nullptr, 0);
        g_rng = strtoull(argv[5], nullptr, 0);
        g_rng_n = n;
        // the reference loop kicks after every accept/revert and then tests
        // its stop rule: stop it on the 2nd draw of kick number kicks+1
        g_stop_after_calls = 2 * (kicks + 1);
        g_on_stop = stop_probe;
        IlsProbe p(c.data(), &args, n);
        g_probe = &p;
        p.optimize(r, 0);
        g_probe = nullptr;
        std::vector<ROUTE_DATA_TYPE> b = IlsProbe::best();
        put_u64(out, IlsProbe::bestLength());
        put_route(out, b);
        put_u64(out, g_log.size() / 3);
    } else if (cmd == "nn") {  // kd-tree nearest-neighbour start tour
        constructKDTree(c.data(), n);
        std::vector<ROUTE_DATA_TYPE> t = initRoute_KD_NN(n, c.data());
        put_route(out, t);
    } else if (cmd == "mf") {  // multiple-fragment (greedy edge) start tour
        constructKDTree(c.data(), n);
        std::vector<ROUTE_DATA_TYPE> t = multipleFragment_KD(n, c.data());
        put_route(out, t);
    } else {
        fclose(out);
        return 2;
    }
    fclose(out);
    return 0;
}
