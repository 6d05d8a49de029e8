// Device self-checks of arithmetic shortcuts against CUDA's own operations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/fsr.h"
#include "fsr_common.cuh"

namespace {

// Every float a in [0, hi] (by bit pattern): div_exact(a, b, RN(1/b)) must
// equal __fdiv_rn(a, b).
__global__ void k_check_division(uint32_t hi_bits, float b, float rb, unsigned long long* bad,
                                 unsigned long long* first_bad)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= hi_bits; i += stride) {
        const float a = __uint_as_float((uint32_t)i);
        const float x = fsr::div_exact(a, b, rb);
        const float y = __fdiv_rn(a, b);
        if (__float_as_uint(x) != __float_as_uint(y)) {
            ++local;
            atomicMin(first_bad, (unsigned long long)i);
        }
    }
    if (local) atomicAdd(bad, local);
}

// Every float x in (0, 1]: spiky_grad must equal float(k x x) in double.
__global__ void k_check_spiky(double k, float khi, float klo, unsigned long long* bad, unsigned long long* first_bad)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t one = 0x3F800000u;
    unsigned long long local = 0;
    for (uint64_t i = 1 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= one; i += stride) {
        const float x = __uint_as_float((uint32_t)i);
        const float a = fsr::spiky_grad(x, khi, klo, k);
        const float b = __double2float_rn(__dmul_rn(__dmul_rn(k, (double)x), (double)x));
        if (__float_as_uint(a) != __float_as_uint(b)) {
            ++local;
            atomicMin(first_bad, (unsigned long long)i);
        }
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace

extern "C" fsr_status fsr_check_spiky_grad(double k, uint64_t* n_checked, uint64_t* n_mismatch)
{
    if (!(k < 0.0) || !(-k >= 1e-20 && -k <= 1e30) || !n_checked || !n_mismatch) return FSR_ERR_INVALID_ARGUMENT;
    const float khi = (float)(-k), klo = (float)(-k - (double)khi);
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return FSR_ERR_CUDA;
    const unsigned long long init[2] = {0ull, ~0ull};
    cudaError_t e = cudaMemcpy(d, init, 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        k_check_spiky<<<sms * 8, 256>>>(k, khi, klo, d, d + 1);
        e = cudaGetLastError();
    }
    unsigned long long out[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(out, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return FSR_ERR_CUDA;
    *n_checked = 0x3F800000ull;
    *n_mismatch = out[0];
    return FSR_OK;
}

extern "C" fsr_status fsr_check_division(float b, uint64_t* n_checked, uint64_t* n_mismatch)
{
    if (!(b > 0.0f) || !std::isfinite(b) || !n_checked || !n_mismatch) return FSR_ERR_INVALID_ARGUMENT;
    const float hi = b * 1.01f;
    uint32_t hi_bits;
    std::memcpy(&hi_bits, &hi, 4);
    const float rb = 1.0f / b;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return FSR_ERR_CUDA;
    const unsigned long long init[2] = {0ull, ~0ull};
    cudaError_t e = cudaMemcpy(d, init, 16, cudaMemcpyHostToDevice);
    int sms = 1;
    if (e == cudaSuccess) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        k_check_division<<<sms * 8, 256>>>(hi_bits, b, rb, d, d + 1);
        e = cudaGetLastError();
    }
    unsigned long long out[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(out, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return FSR_ERR_CUDA;
    *n_checked = (uint64_t)hi_bits + 1;
    *n_mismatch = out[0];
    return FSR_OK;
}

namespace {

// Independent FMA chains per thread: the FP32 pipe's issue rate, not its
// latency, bounds the kernel.  The result is stored only when it is 0 (it
// never is for these inputs) so that the chains are not removed.
__global__ void __launch_bounds__(256) k_fma_rate(float a, float b, int iters, float* sink)
{
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (float)(threadIdx.x + k) * 1e-3f + 1.0f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r)
#pragma unroll
            for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 0.0f) *sink = s;
}

}  // namespace

extern "C" fsr_status fsr_measure_fp32_rate(int device, double* tflops)
{
    if (!tflops) return FSR_ERR_INVALID_ARGUMENT;
    *tflops = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) return FSR_ERR_CUDA;
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) return FSR_ERR_OUT_OF_MEMORY;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const unsigned blocks = (unsigned)sms * 8;  // 8 blocks of 256 threads per SM: every warp slot busy
    const int iters = 4096;
    double best = 0.0;
    // the multiplier keeps every chain bounded: x -> x a + b with |a| < 1
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        k_fma_rate<<<blocks, 256>>>(0.999f, 1e-3f, iters, sink);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8 * 16 * (double)iters * 256.0 * blocks;
        if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return FSR_ERR_CUDA;
    *tflops = best;
    return FSR_OK;
}
