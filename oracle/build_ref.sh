#!/bin/sh
# Builds oracle/_ref/libacumref_f32.so and oracle/_ref/libacumref_f64.so from the
# reference's own sources, read in place (they are never copied into this repository).
#
#   libacumref_f32.so  the sources as written (float storage), host C++
#   libacumref_f64.so  the same sources with `float` promoted to `double` (ref_shim.h),
#                      i.e. the FP64 build that the plain tonal form is held to
#   core_sm103a.cubin  the reference's tonal kernel (core.cu) for the GPU (oracle/ref_gpu.py
#                      times it there)
#
# TEST INFRASTRUCTURE ONLY.  Only the tests, the smoke check and bench.py's CPU baseline
# leg may load these libraries.  They are built from the reference source tree in place;
# on a machine without that tree the script exits 0 and builds nothing.  The tree is
# ACUM_REF_DIR when that is set, else the location this recipe was written for.
#
# Flags: -ftrivial-auto-var-init=zero makes the uninitialised locals of bb_core.cu
# (notably `aa` in the convected-time formula at bb_core.cu:520) read as zero instead of
# stack garbage; -ffp-contract=off keeps a*b+c unfused so results do not depend on the
# host's FMA support.  main.cu is not compiled (it holds the <<<>>> launch and CUDA
# allocation); ref_harness.cpp replays its sequence instead.
set -e
REF="${ACUM_REF_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/core.cu" ]; then
    echo "build_ref: reference sources not found at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
SRCS="variables.cu io.cu mathfunc.cu preprocess.cu core.cu bb_core.cu bb_utils.cu"
FILES=""
for s in $SRCS; do FILES="$FILES $REF/$s"; done
CXX="${CXX:-g++}"
COMMON="-O2 -fPIC -shared -w -ffp-contract=off -ftrivial-auto-var-init=zero -I$REF -include $HERE/ref_shim.h"
$CXX $COMMON -x c++ $FILES "$HERE/ref_harness.cpp" -o "$OUT/libacumref_f32.so.tmp" &
P1=$!
$CXX $COMMON -DACUM_REF_F64 -x c++ $FILES "$HERE/ref_harness.cpp" -o "$OUT/libacumref_f64.so.tmp" &
P2=$!
wait $P1
wait $P2
mv "$OUT/libacumref_f32.so.tmp" "$OUT/libacumref_f32.so"
mv "$OUT/libacumref_f64.so.tmp" "$OUT/libacumref_f64.so"
echo "build_ref: built $OUT/libacumref_f32.so $OUT/libacumref_f64.so"
# The reference's own tonal kernel (core.cu:18) for the GPU, unmodified: a cubin for sm_103a.
NVCC="${NVCC:-nvcc}"
if command -v "$NVCC" > /dev/null 2>&1; then
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -I"$REF" "$REF/core.cu" -o "$OUT/core_sm103a.cubin"
    echo "build_ref: built $OUT/core_sm103a.cubin"
fi
