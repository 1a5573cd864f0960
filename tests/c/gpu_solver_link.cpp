// Link check of integration/GPUSolver.h: compiled against the reference's
// own headers (src/solvers/twoOptLocalSolver.h, localSolver.h, defs.h) and
// linked with the reference's twoOptLocalSolver.cpp and common.c and with
// liblogo_gpu.so.  Run without arguments it only proves that every symbol
// resolves; with "descend" it builds a GPUSolver on device 0 and descends a
// crossed 4-city tour through the reference's interface.
#include <cstring>

#include "GPUSolver.h"

int main(int argc, char **argv) {
    if (argc < 2 || std::strcmp(argv[1], "descend") != 0) return 0;
    static city_coords c[4] = {{0, 0}, {10, 0}, {10, 10}, {0, 10}};
    cmdArguments args;
    std::memset(&args, 0, sizeof(args));
    GPUSolver s(c, &args, "gpu", 0, 4);
    vector<ROUTE_DATA_TYPE> route = {0, 2, 1, 3};
    vector<unsigned long> best;
    s.optimize(route, best);
    for (size_t k = 0; k < route.size(); ++k) printf("%u ", (unsigned)route[k]);
    printf("\n");
    return 0;
}
