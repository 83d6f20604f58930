#!/usr/bin/env bash
# oracle/build_ref.sh — TEST INFRASTRUCTURE ONLY.
#
# Builds the checkers made from the reference's own code. Every output goes to
# oracle/_ref/, which is never committed.
#
# 1. Where the reference tree is named by RHIZOME_REFERENCE and present:
#    * oracle/_ref/libref_math.so — the reference's host/device geometry primitives
#      (native/src/core/math_utils.cuh) compiled on the host with g++, through the
#      project-written glm stand-in in oracle/ref_shim/;
#    * oracle/_ref/src/ — an unmodified copy of the seven reference files the fast-SDF
#      translation unit needs (the include closure of
#      native/src/engine/sdf/cuda_rasterizer.cu), and oracle/_ref/assets/mug.obj, the
#      reference's own specimen. The copy travels with the working tree to a GPU host
#      that holds no reference tree, so the reference's GPU code can be compiled there.
# 2. Wherever oracle/_ref/src/ and nvcc are present (here and on a GPU host):
#    * oracle/_ref/libref_rast.so — oracle/ref_gpu_harness.cu, which #includes the
#      reference's cuda_rasterizer.cu, compiled with the reference's own nvcc flags
#      (native/CMakeLists.txt:9-11, 33-36, CMake's Release -O3; FMA contraction left at
#      nvcc's default, on), for sm_103a.
# Exits 0 when a step's inputs are absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${RHIZOME_REFERENCE:-}"
REF_SRC="$REF_ROOT/native/src"
OUT="$HERE/_ref"
STAGE="$OUT/src"
CLOSURE="engine/sdf/cuda_rasterizer.cu engine/sdf/cuda_rasterizer.hpp engine/sdf/cuda_types.hpp
engine/sdf/cuda_common.cuh engine/io/mesh.hpp core/math_utils.cuh core/unified_logger.hpp"

if [ -n "$REF_ROOT" ] && [ -f "$REF_SRC/core/math_utils.cuh" ]; then
  mkdir -p "$OUT"
  g++ -O2 -std=c++20 -ffp-contract=off -fPIC -shared \
    -I "$HERE/ref_shim" -I "$REF_SRC" \
    "$HERE/ref_math_wrap.cpp" -o "$OUT/libref_math.so"
  echo "built $OUT/libref_math.so"
  for f in $CLOSURE; do
    mkdir -p "$STAGE/$(dirname "$f")"
    cp -p "$REF_SRC/$f" "$STAGE/$f"
  done
  if [ -f "$REF_ROOT/native/assets/mug.obj" ]; then
    mkdir -p "$OUT/assets"
    cp -p "$REF_ROOT/native/assets/mug.obj" "$OUT/assets/mug.obj"
  fi
  echo "staged the reference's fast-SDF sources in $STAGE"
else
  echo "RHIZOME_REFERENCE unset or not a reference tree; libref_math.so not built, sources not staged"
fi

NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
LIB="$OUT/libref_rast.so"
HARNESS="$HERE/ref_gpu_harness.cu"
if [ -f "$STAGE/engine/sdf/cuda_rasterizer.cu" ] && [ -x "$NVCC" ]; then
  stale=1
  if [ -f "$LIB" ]; then
    stale=0
    for dep in "$HARNESS" "$HERE/ref_shim/glm/glm.hpp" "$STAGE"/engine/sdf/* "$STAGE"/engine/io/* "$STAGE"/core/*; do
      if [ "$dep" -nt "$LIB" ]; then stale=1; fi
    done
    # a library built on another host architecture is rebuilt
    if [ "$(cat "$LIB.arch" 2>/dev/null)" != "$(uname -m)" ]; then stale=1; fi
  fi
  if [ "$stale" = 1 ]; then
    "$NVCC" -std=c++20 --extended-lambda --expt-relaxed-constexpr -O3 -DNDEBUG \
      -gencode arch=compute_103a,code=sm_103a -Xcompiler -fPIC -shared \
      -I "$HERE/ref_shim" -I "$STAGE" "$HARNESS" -o "$LIB"
    uname -m > "$LIB.arch"
    echo "built $LIB"
  fi
else
  echo "staged reference sources or nvcc absent; libref_rast.so not built"
fi
