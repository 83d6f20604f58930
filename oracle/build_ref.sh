#!/usr/bin/env bash
# oracle/build_ref.sh — TEST INFRASTRUCTURE ONLY.
# Builds oracle/_ref/libref_math.so from the reference's own sources where they lie
# (native/src/core/math_utils.cuh, native/src/engine/sdf/cuda_types.hpp) plus the
# project-written glm stand-in. Output goes only to oracle/_ref/. Exits 0 without
# building when the reference tree is absent (e.g. on the GPU host).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_SRC="${RHIZOME_REFERENCE:-/root/reference}/native/src"
if [ ! -f "$REF_SRC/core/math_utils.cuh" ]; then
  echo "reference tree not present; oracle/_ref not built"
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++20 -ffp-contract=off -fPIC -shared \
  -I "$HERE/ref_shim" -I "$REF_SRC" \
  "$HERE/ref_math_wrap.cpp" -o "$HERE/_ref/libref_math.so"
echo "built $HERE/_ref/libref_math.so"
