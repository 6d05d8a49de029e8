#!/usr/bin/env bash
# Oracle recipe: compile the reference's own kernel bodies and host marching
# cubes as a host shared library, oracle/_ref/libfsr_refkernels.so.
#
# Reads the reference sources where they lie and writes only object code
# into oracle/_ref/ (git-ignored).  It never runs the reference's own build
# system.  Test infrastructure only.
#
# The reference checkout is REF_ROOT; unset, it is the build container's
# checkout location below.  `build_ref.sh --print-root` prints the resolved
# root (the drop-in link test and the golden-vector script ask it), and the
# recipe exits 2 when no reference sources are there (the GPU machines have
# none: they use what was built before).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
if [ "${1:-}" = "--print-root" ]; then
  echo "$REF_ROOT"
  exit 0
fi
GPU_DIR="$REF_ROOT/FluidSurfaceReconstruction/GPU"
OUT="$HERE/_ref"
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
if [ ! -f "$GPU_DIR/ReconstructionCUDA.cu" ]; then
  echo "build_ref: reference sources not found under $REF_ROOT" >&2
  exit 2
fi
mkdir -p "$OUT"
rm -f "$OUT/ref_kernels.inc"
# kernel bodies only: cu lines 28-1008 (tables, helpers, all per-stage
# kernels) and 1354-1396 (hash kernels); launchers and thrust calls excluded.
# The extract lives in a temporary directory: no reference source is kept.
TMP="$(mktemp -d)"
trap 'rm -rf "$TMP"' EXIT
sed -n '28,1008p;1354,1396p' "$GPU_DIR/ReconstructionCUDA.cu" > "$TMP/ref_kernels.inc"
CXX="${CXX:-g++}"
FLAGS=(-std=c++14 -O2 -fPIC -fopenmp -ffp-contract=off -fno-fast-math -w
       -I"$HERE/ref_shim" -I"$HERE" -I"$TMP" -I"$GPU_DIR" -I"$REF_ROOT/include" -I"$CUDA_INC"
       -include "$HERE/ref_shim/fsr_ref_emul.h")
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o"
"$CXX" "${FLAGS[@]}" -c "$GPU_DIR/MarchingCubesCPU.cpp" -o "$OUT/MarchingCubesCPU.o"
"$CXX" "${FLAGS[@]}" -c "$GPU_DIR/MarchingCubesHelper.cpp" -o "$OUT/MarchingCubesHelper.o"
"$CXX" "${FLAGS[@]}" -c "$GPU_DIR/MathVector.cpp" -o "$OUT/MathVector.o"
"$CXX" -shared -fopenmp -o "$OUT/libfsr_refkernels.so" "$OUT"/ref_driver.o \
  "$OUT"/MarchingCubesCPU.o "$OUT"/MarchingCubesHelper.o "$OUT"/MathVector.o
echo "build_ref: wrote $OUT/libfsr_refkernels.so"
