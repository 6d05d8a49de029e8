/*
 * Host emulation layer for compiling the reference's CUDA kernel bodies
 * (FluidSurfaceReconstruction/GPU/ReconstructionCUDA.cu, kernels only) as
 * plain C++ with g++.  TEST INFRASTRUCTURE ONLY: this header is part of the
 * oracle recipe and is never linked into the product library.
 *
 * What it provides:
 *  - execution-space qualifiers defined away (__global__, __device__, ...),
 *    defined before any CUDA header so the CUDA headers keep them empty;
 *  - per-OS-thread launch coordinates (blockIdx, threadIdx, blockDim,
 *    gridDim) that a host launcher sets before calling a kernel body;
 *  - a minimal stand-in for the legacy texture-reference API used by the
 *    marching-cubes table lookups (ReconstructionCUDA.cu:29-37, 50-65):
 *    a texture is a plain table pointer and tex1Dfetch an array read;
 *  - host versions of the IEEE round-to-nearest intrinsics the vendored SVD
 *    header uses, written from their IEEE definitions (single rounding of the
 *    exact result): add and subtract are plain float ops when FP contraction
 *    is off; the reciprocal square root is evaluated in double and rounded;
 *  - float and unsigned overloads of max/min (CUDA device code resolves
 *    max(float,float) to the float function; the host helper header only
 *    defines int ones).
 */
#pragma once

#define __global__
#define __device__
#define __host__
#define __shared__
#define __constant__
#define __forceinline__ inline
#define __DEVICE_LAUNCH_PARAMETERS_H__ 1

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <fstream>
#include <algorithm>
#include <vector_types.h>
#include <vector_functions.h>
#include <driver_types.h>
#include <texture_types.h>

extern thread_local uint3 blockIdx;
extern thread_local uint3 threadIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

template <class T, int Dim, enum cudaTextureReadMode Mode>
struct texture { const T* table = nullptr; };

template <class T, int Dim, enum cudaTextureReadMode Mode>
inline T tex1Dfetch(const texture<T, Dim, Mode>& t, int i) { return t.table[i]; }

template <class T, int Dim, enum cudaTextureReadMode Mode>
inline cudaError_t cudaBindTexture(size_t* /*offset*/, texture<T, Dim, Mode>& t,
                                   const void* p, const cudaChannelFormatDesc& /*desc*/)
{
    t.table = static_cast<const T*>(p);
    return cudaSuccess;
}

inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __frsqrt_rn(float x) { return (float)(1.0 / std::sqrt((double)x)); }

inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
