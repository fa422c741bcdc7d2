#!/bin/sh
# Builds the reference's own fractal code into oracle/_ref/ (git-ignored).
#
# TEST INFRASTRUCTURE ONLY.  Run where the reference checkout exists:
# REFERENCE_ROOT names it (oracle/build_oracle.py sets it: $REFERENCE_ROOT, else
# a checkout named `reference` beside this repository).  Steps:
#   1. copy the few CUDA sources the path needs into oracle/_ref/src/ (a
#      build-directory copy; the checkout is read-only), patching one token in
#      fractalRendererGeneric.cu:200 that current nvcc rejects
#      (relative_in_old.cast<float>() -> relative_in_old.template cast<float>());
#   2. host build of computeFractal/colorize (oracle/ref_host.cpp) ->
#      oracle/_ref/libchaos_ref.so, with -ffp-contract=off;
#   3. sm_103a cubins of the reference modules, default arithmetic and
#      --fmad=false: oracle/_ref/ref_<fractal>.cubin, ref_<fractal>_nofma.cubin.
# Steps 2-3 also run from an existing oracle/_ref/src/ when the checkout is absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
REF="${REFERENCE_ROOT:?REFERENCE_ROOT must name the chaos-ultra checkout}"
C="$REF/src/main/cuda"
mkdir -p "$OUT/src/fractals"
if [ -f "$C/fractalRendererGeneric.cu" ]; then
  cp "$C/helpers.cuh" "$OUT/src/helpers.cuh"
  for f in fractal.cuh mandelbrot.cu julia.cu newton_wired.cu newton_generic.cu newton_iterations.cu; do
    cp "$C/fractals/$f" "$OUT/src/fractals/$f"
  done
  sed 's/relative_in_old\.cast<float>()/relative_in_old.template cast<float>()/' \
    "$C/fractalRendererGeneric.cu" > "$OUT/src/fractalRendererGeneric.cu"
fi
if [ ! -f "$OUT/src/fractalRendererGeneric.cu" ]; then
  echo "build_ref.sh: reference sources not found (REFERENCE_ROOT=$REF)" >&2
  exit 3
fi
CXX="${CXX:-g++}"
# -Dlb=lt -Drt=rb: the Rectangle(Point lt, Point rb) constructor at helpers.cuh:83
# names lb/rt, which do not exist; nvcc never instantiates it, g++ parses it.
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
"$CXX" -O2 -ffp-contract=off -fopenmp -fPIC -shared -DNDEBUG -Dlb=lt -Drt=rb \
  -I"$HERE" -I"$OUT/src" -I"$CUDA_INC" -I"$CUDA_INC/cccl" "$HERE/ref_host.cpp" -o "$OUT/libchaos_ref.so"
if [ "${SKIP_CUBIN:-0}" != "1" ]; then
  NVCC="${NVCC:-nvcc}"
  for f in mandelbrot julia newton_wired newton_generic newton_iterations; do
    printf '#include "fractals/%s.cu"\n#include "fractalRendererGeneric.cu"\n' "$f" > "$OUT/src/ref_$f.cu"
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -DNDEBUG -I"$OUT/src" \
      "$OUT/src/ref_$f.cu" -o "$OUT/ref_$f.cubin" &
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -DNDEBUG --fmad=false -I"$OUT/src" \
      "$OUT/src/ref_$f.cu" -o "$OUT/ref_${f}_nofma.cubin" &
  done
  wait
  for f in mandelbrot julia newton_wired newton_generic newton_iterations; do
    [ -s "$OUT/ref_$f.cubin" ] && [ -s "$OUT/ref_${f}_nofma.cubin" ] || { echo "cubin build failed" >&2; exit 4; }
  done
fi
echo "build_ref.sh: ok"
