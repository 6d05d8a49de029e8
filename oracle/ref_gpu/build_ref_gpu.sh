#!/usr/bin/env bash
# Oracle recipe: the reference's own CUDA kernels, built for sm_103a as a
# device-code module (cubin), oracle/_ref/ref_kernels_sm103a.cubin.
# Test and measurement infrastructure only: the GPU baseline leg of bench.py
# and tests/test_gpu_reference_build.py load it through
# oracle/ref_gpu/ref_launchers.cu.
#
# The reference targets CUDA 10.1; CUDA 13 removed texture references, so a
# patched copy of ReconstructionCUDA.cu/.cuh is compiled, in a temporary
# directory (nothing of the reference is kept):
#   * the four marching-cubes table textures become __device__ table
#     pointers (texture<T,1,...> X -> __device__ const T* X; tex1Dfetch(X, i)
#     -> X[i]; cudaBindTexture -> cudaMemcpyToSymbol of the pointer), so the
#     table loads go through ld.global instead of the texture path;
#   * the two __constant__ definitions move from the .cu into the header as
#     static definitions (extern __constant__ needs relocatable device code);
#   * an empty Windows.h and the oracle's two-macro helper_cuda.h stand in
#     for the Windows header and the CUDA-10 samples header.
# Everything else, every kernel body included, is the reference's source as
# it lies.  The reference checkout is REF_ROOT (see oracle/build_ref.sh);
# the recipe exits 2 when it is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ORACLE="$(dirname "$HERE")"
REF_ROOT="$(bash "$ORACLE/build_ref.sh" --print-root)"
GPU_DIR="$REF_ROOT/FluidSurfaceReconstruction/GPU"
OUT="$ORACLE/_ref"
if [ ! -f "$GPU_DIR/ReconstructionCUDA.cu" ]; then
  echo "build_ref_gpu: reference sources not found under $REF_ROOT" >&2
  exit 2
fi
NVCC="${CUDA_HOME:-/usr/local/cuda}/bin/nvcc"
mkdir -p "$OUT"
TMP="$(mktemp -d)"
trap 'rm -rf "$TMP"' EXIT
mkdir -p "$TMP/inc"
: > "$TMP/inc/Windows.h"
perl -pe '
  s/^\s*__constant__\s+float\s+(EPSILON_|SIGMA)\s*=.*$//;
  s/^texture\s*<\s*(\w+)\s*,\s*1\s*,\s*cudaReadModeElementType\s*>\s*(\w+)\s*;/__device__ const $1* $2;/;
  s/tex1Dfetch\((\w+),\s*([^;]*?)\)(\s*;)/$1\[$2\]$3/g;
  s/cudaBindTexture\(0,\s*(\w+),\s*(\w+),\s*\w+\)/cudaMemcpyToSymbol($1, &$2, sizeof(void*))/;
' "$GPU_DIR/ReconstructionCUDA.cu" > "$TMP/ReconstructionCUDA.cu"
perl -pe '
  s/^extern "C" __constant__ float SIGMA;/static __constant__ float SIGMA = 315.0f \/ (64.0f * 3.1415926535898f);/;
  s/^extern "C" __constant__ float EPSILON_;/static __constant__ float EPSILON_ = (float)1.0e-7;/;
' "$GPU_DIR/ReconstructionCUDA.cuh" > "$TMP/ReconstructionCUDA.cuh"
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -w \
  -I"$TMP" -I"$TMP/inc" -I"$ORACLE/ref_shim" -I"$GPU_DIR" -I"$REF_ROOT/include" \
  -include fstream -include memory \
  "$TMP/ReconstructionCUDA.cu" -o "$OUT/ref_kernels_sm103a.cubin"
echo "build_ref_gpu: wrote $OUT/ref_kernels_sm103a.cubin"
