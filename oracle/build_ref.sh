#!/usr/bin/env bash
# Recipe for oracle/_ref: the reference's own CPU code for the omni path, compiled from
# its sources, used only to pin the oracle and as the timed CPU baseline.
#
#   stage  (needs the reference tree, located by REF_ROOT, which has no default):
#          copies the reference functions on the hot path, by line range, from
#          Omni3D_8.0/Omni3D_8.0/kernel.cu, plus sor3D.cpp, calRHS.cpp,
#          initialIntegration.cpp and the direction files GridIcosahedronDivide{2,3,4}.dat
#          of Omni3D_8.0/Executable, into
#          oracle/_ref/src/ (git-ignored build intermediates, never committed).
#   build  compiles oracle/_ref/src/* with oracle/ref_driver.cpp into
#          oracle/_ref/libomni_ref.so.  Runs wherever oracle/_ref/src exists, so a
#          staged tree can be rebuilt on a machine without the reference.
#
# Line ranges of kernel.cu (reference file:line):
#   119-1113   ntoijk, crosspoint, cross2point
#   1743-3085  bodyIntegralInner and its variants (StepCount, Weighted, WeightedFixedBC,
#              Select, SelectFixedBC, MiniCurl, WeightedMiniCurl)
#   8171-8212  calIndex
#   8271-8378  omni3dparallellinesESInnerCPU, devidecountCPU, devidecountInnerCPU,
#              calCurlofMaterialAccCPU
# calRHS.cpp line 10 re-allocates the caller's output buffer (RHS = new double[...]),
# which drops the result; the staged copy omits that one line.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
REF_ROOT="${REF_ROOT:-}"
K="$REF_ROOT/Omni3D_8.0/Omni3D_8.0"
CXX="${CXX:-g++}"
what="${1:-all}"

stage() {
    [ -n "$REF_ROOT" ] || { echo "build_ref: set REF_ROOT to the reference checkout to stage its sources" >&2; return 1; }
    [ -f "$K/kernel.cu" ] || { echo "build_ref: reference not found at $K" >&2; return 1; }
    mkdir -p "$SRC/stub"
    {
        echo '// staged by oracle/build_ref.sh from the reference kernel.cu (line ranges in the recipe)'
        echo '#include <cmath>'
        echo '#include <cstdio>'
        echo '#include <cstdlib>'
        echo '#include <cstring>'
        echo 'using namespace std;'
        echo '#define __device__'
        echo '#define __host__'
        echo '#define __global__'
        echo '#define zero 1e-7'
        echo '#define PI 3.1415926535897932384626433832795'
        for r in 119,1113 1743,3085 8171,8212 8271,8378; do
            sed -n "${r}p" "$K/kernel.cu" | tr -d '\r'
        done
    } > "$SRC/ref_kernel_extract.cpp"
    tr -d '\r' < "$K/sor3D.cpp" > "$SRC/sor3D.cpp"
    tr -d '\r' < "$K/sor3D.h" > "$SRC/sor3D.h"
    tr -d '\r' < "$K/calRHS.cpp" | sed '10d' > "$SRC/calRHS.cpp"
    tr -d '\r' < "$K/calRHS.h" > "$SRC/calRHS.h"
    tr -d '\r' < "$K/initialIntegration.cpp" > "$SRC/initialIntegration.cpp"
    tr -d '\r' < "$K/initialIntegration.h" > "$SRC/initialIntegration.h"
    printf '#include <cstring>\n#include <cstdlib>\n#include <cmath>\n' > "$SRC/stub/afx.h"
    for lv in 2 3 4; do
        cp "$REF_ROOT/Omni3D_8.0/Executable/GridIcosahedronDivide$lv.dat" "$SRC/"
    done
    # the staged files must still hold the functions the driver binds
    grep -q 'bool cross2point' "$SRC/ref_kernel_extract.cpp"
    grep -q 'float bodyIntegralInner(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'float bodyIntegralInnerSelect(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'float bodyIntegralInnerWeighted(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'float bodyIntegralInnerWeightedFixedBC(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'float bodyIntegralInnerSelectFixedBC(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'float bodyIntegralInnerMiniCurl(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'float bodyIntegralInnerWeightedMiniCurl(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'void calIndex(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'void calCurlofMaterialAccCPU(' "$SRC/ref_kernel_extract.cpp"
    grep -q 'RHS=new double' "$SRC/calRHS.cpp" && { echo "build_ref: calRHS patch failed" >&2; return 1; }
    echo "staged reference sources in $SRC"
}

build() {
    [ -f "$SRC/ref_kernel_extract.cpp" ] || { echo "build_ref: nothing staged in $SRC" >&2; return 1; }
    # -ffp-contract=off: the reference's float expressions are evaluated one rounding per
    # operation (MSVC x64 default); aarch64 gcc would otherwise fuse multiply-adds.
    local FLAGS="-O2 -fPIC -ffp-contract=off -fopenmp -w"
    "$CXX" $FLAGS -c "$SRC/ref_kernel_extract.cpp" -o "$OUT/ref_kernel_extract.o"
    "$CXX" $FLAGS -I"$SRC/stub" -I"$SRC" -c "$SRC/sor3D.cpp" -o "$OUT/sor3D.o"
    "$CXX" $FLAGS -I"$SRC/stub" -I"$SRC" -c "$SRC/calRHS.cpp" -o "$OUT/calRHS.o"
    "$CXX" $FLAGS -I"$SRC/stub" -I"$SRC" -c "$SRC/initialIntegration.cpp" -o "$OUT/initialIntegration.o"
    "$CXX" $FLAGS -Wall -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o"
    "$CXX" -shared -fopenmp -o "$OUT/libomni_ref.so" "$OUT/ref_driver.o" "$OUT/ref_kernel_extract.o" \
        "$OUT/sor3D.o" "$OUT/calRHS.o" "$OUT/initialIntegration.o"
    echo "built $OUT/libomni_ref.so"
}

case "$what" in
    stage) stage ;;
    build) build ;;
    all) stage && build ;;
    *) echo "usage: $0 [stage|build|all]" >&2; exit 2 ;;
esac
