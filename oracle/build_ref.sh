#!/usr/bin/env bash
# Compile the reference's own CPU imaging library (libcpu_imaging32.so / libcpu_imaging64.so)
# from its sources where they lie, into oracle/_ref/.  TEST INFRASTRUCTURE ONLY: the result
# is the parity oracle that pins oracle/bullseye_oracle.c and generates tests/golden/
# fixtures.  It is never linked into, or called by, the product.
#
# Flags follow the reference's CMake recipe (bullseye/mo/cpu_algorithm/single/CMakeLists.txt:18):
# -O3 -fopenmp -pthread -std=c++11 -fno-strict-aliasing, scalar path (VECTORIZE=OFF).
# Shims (oracle/shim): empty casacore/boost headers (included but unused by the reference)
# and an FFTW-API header implemented by oracle/fftw_shim.c (FFTW is absent from this image).
# cufft.h is only needed for the __host__/__device__ macros (cu_common.h:41).
#
# Usage: oracle/build_ref.sh [reference_root]
# The reference root is the argument, else $BULLSEYE_REFERENCE, else the read-only mount where
# this build environment keeps the reference (this recipe is the one place that names it).
# Exits 0 without building when the reference tree is absent (e.g. on a machine that only
# has this repository).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${BULLSEYE_REFERENCE:-/root/reference}}"
MO="$REF/bullseye/mo"
if [ ! -f "$MO/cpu_algorithm/wrapper.cpp" ]; then
    echo "build_ref: reference sources not found under $REF; skipping oracle/_ref" >&2
    exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
gcc -O2 -fPIC -c "$HERE/fftw_shim.c" -o "$OUT/fftw_shim.o"
build() {
    local prec="$1" name="$2"
    g++ -DBULLSEYE_"$prec" -fPIC -shared -O3 -fopenmp -pthread -std=c++11 -fno-strict-aliasing -w \
        -I"$HERE/shim" -I"$MO/cpu_gpu_common" -I"$MO/cpu_algorithm" -I"$CUDA_INC" \
        "$MO/cpu_algorithm/wrapper.cpp" \
        "$MO/cpu_gpu_common/fft_shift_utils.cpp" \
        "$MO/cpu_gpu_common/fft_and_repacking_routines.cpp" \
        "$OUT/fftw_shim.o" -o "$OUT/$name"
}
# the nearest-neighbour sampling-count harness (oracle/ref_nn_harness.cpp) over the same headers
build_nn() {
    local prec="$1" name="$2"
    g++ -DBULLSEYE_"$prec" -fPIC -shared -O3 -fopenmp -pthread -std=c++11 -fno-strict-aliasing -w \
        -I"$HERE/shim" -I"$MO/cpu_gpu_common" -I"$MO/cpu_algorithm" -I"$CUDA_INC" \
        "$HERE/ref_nn_harness.cpp" -o "$OUT/$name"
}
build SINGLE libcpu_imaging32.so &
build DOUBLE libcpu_imaging64.so &
build_nn SINGLE libref_nn32.so &
build_nn DOUBLE libref_nn64.so &
wait
echo "build_ref: built $OUT/libcpu_imaging32.so $OUT/libcpu_imaging64.so $OUT/libref_nn32.so $OUT/libref_nn64.so"
