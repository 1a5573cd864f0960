#!/bin/sh
# Compiles the reference's own C++ sources for the 2-opt path, in place under
# the reference checkout, together with oracle/ref_harness.cpp into
# oracle/_ref/ref_harness (TEST INFRASTRUCTURE ONLY: it pins the oracle).
#
# Needs the reference checkout (REF, default /root/reference) and an x86-64
# host: the reference CPU solver uses AVX intrinsics (src/utils/cpusimd.h).
# Elsewhere it exits 0 without building; the tests that need it skip.
#
# Flags follow the reference Makefile (Makefile:80-81,116-125) except:
#  -ffp-contract=off and no -march=native, so that sqrtf(dx*dx+dy*dy) is not
#  contracted into an FMA (the canonical per-edge distance);
#  ref_rand_hook.h force-included into ILSGlobalSolver.cpp only, so kicks draw from a
#  seeded SplitMix64 defined in the harness.
set -e
REF=${REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
    echo "build_ref: no reference checkout at $REF; skipped"
    exit 0
fi
case "$(uname -m)" in
    x86_64) ;;
    *) echo "build_ref: reference CPU solver needs x86 AVX; skipped"; exit 0 ;;
esac
mkdir -p "$OUT"
CXX=${CXX:-g++}
INC="-I$REF/src/solvers -I$REF/src/utils -I$REF/src -I$REF/src/parser -I$REF/src/kdtree++"
FLAGS="-std=gnu++11 -O2 -ffp-contract=off -mavx -fpermissive -w -DUSE_CPU_SIMD -DUSE_AVX \
 -DHAVE_PTHREADS -DDEFAULT_MAX_CORES=8 -DHOST=ref $INC"
objs=""
for src in solvers/twoOptLocalSolver.cpp solvers/ILSGlobalSolverSequential.cpp \
           solvers/cpuSolver.cpp solvers/cpuMTSolver.cpp utils/common.c \
           utils/kdtree_utils.c utils/construction.c utils/tsp_loader.c; do
    o="$OUT/$(basename "$src" | sed 's/\.[a-z]*$//').o"
    $CXX $FLAGS -x c++ -c "$REF/src/$src" -o "$o" &
    objs="$objs $o"
done
$CXX $FLAGS -include "$HERE/ref_rand_hook.h" -x c++ -c "$REF/src/solvers/ILSGlobalSolver.cpp" \
    -o "$OUT/ILSGlobalSolver.o" &
$CXX $FLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" &
wait
$CXX -o "$OUT/ref_harness" $objs "$OUT/ILSGlobalSolver.o" "$OUT/ref_harness.o" -lpthread
echo "build_ref: built $OUT/ref_harness"
