#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure): oracle/_build/liboracle32.so
# (reference FP32 semantics), liboracle64.so (FP64 continuous values) and
# libio_port.so (the reference's stream-based .xyz reader and .obj writer,
# the file formats' timing baseline).
# -ffp-contract=off keeps every multiply and add separately rounded, as the
# reference source is written (aarch64 gcc would otherwise fuse them).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_build"
mkdir -p "$OUT"
CC="${CC:-gcc}"
FLAGS=(-std=c11 -O2 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math -Wall -Wno-unknown-pragmas -Wno-unused-but-set-variable)
"$CC" "${FLAGS[@]}" -DFSR_REAL_BITS=32 -o "$OUT/liboracle32.so" "$HERE/fsr_oracle.c" -lm &
P1=$!
"$CC" "${FLAGS[@]}" -DFSR_REAL_BITS=64 -o "$OUT/liboracle64.so" "$HERE/fsr_oracle.c" -lm &
P2=$!
"${CXX:-g++}" -std=c++17 -O2 -fPIC -shared -o "$OUT/libio_port.so" "$HERE/io_port.cpp" &
P3=$!
# the launchers of the reference's own kernels (oracle/ref_gpu): they load
# the cubin that oracle/ref_gpu/build_ref_gpu.sh builds from the reference's
# sources where those are present, and is shipped with the other build
# products elsewhere
NVCC="${CUDA_HOME:-/usr/local/cuda}/bin/nvcc"
"$NVCC" -gencode arch=compute_103a,code=sm_103a -std=c++17 -O2 -Xcompiler -fPIC -shared \
  -I"$(dirname "$HERE")/include" -o "$OUT/libref_gpu.so" "$HERE/ref_gpu/ref_launchers.cu" \
  -L"${CUDA_HOME:-/usr/local/cuda}/lib64/stubs" -lcuda &
P4=$!
wait "$P1"
wait "$P2"
wait "$P3"
wait "$P4"
echo "build_oracle: wrote $OUT/liboracle32.so $OUT/liboracle64.so $OUT/libio_port.so $OUT/libref_gpu.so"
