/* Force-included (-include) into the reference's ILSGlobalSolver.cpp by
 * oracle/build_ref.sh: after the C and C++ library headers are in, rand()
 * in that file resolves to the harness's seeded SplitMix64 draw. */
#include <stdlib.h>
#include <cstdlib>
#include <algorithm>
extern "C" int logo_ref_rand(void);
#define rand logo_ref_rand
