// Device-wide primitives: exclusive prefix sum and stable LSD radix sort.
// Both replace the reference's thrust calls (ReconstructionCUDA.cu:1158
// exclusive_scan, :1463 sort_by_key); neither synchronises the stream and
// sizes may live in device memory, so a frame needs no host round trip.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fsr {

constexpr uint32_t kScanThreads = 256;
constexpr uint32_t kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;  // 4096

// What the scan reads: u32 elements, or the popcount of each u32 word.
enum class ScanInput : int {
    kValue = 0,          // the element
    kPopcount = 1,       // popcount of the element
    kNonzero = 2         // element != 0
};

#ifdef __CUDACC__
// Inclusive scan of one value per thread across the block (256 threads).
__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t x, uint32_t* warp_sums)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < (kScanThreads / 32) ? warp_sums[lane] : 0u;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < (kScanThreads / 32)) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t add = warp ? warp_sums[warp - 1] : 0u;
    return x + add;
}
#endif

// Scratch words needed by scan_u32 for up to n_max elements.
size_t scan_scratch_words(uint64_t n_max);

// out[i] = sum of in'[0..i) where in' is the element transformed per ScanInput.
// Element count: *n_dev when n_dev is not null, else n_host; the count must
// not exceed n_max (the size the launch grid is built for).  *total (may be
// null) receives the sum of all elements.  Aliasing in == out is allowed.
cudaError_t scan_u32(const uint32_t* in, uint32_t* out, uint32_t n_host, const uint32_t* n_dev,
                     uint32_t n_max, uint32_t* total, ScanInput mode, uint32_t* scratch,
                     cudaStream_t stream);

// Stable sort of (key, value) pairs by the low `key_bits` bits of key.  The
// sorted pairs end in (k0, v0) when the function returns 0 and in (k1, v1)
// when it returns 1 (ping-pong buffers).  scratch: radix_scratch_words(n).
size_t radix_scratch_words(uint32_t n);
int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n,
                     uint32_t key_bits, uint32_t* scratch, cudaStream_t stream, cudaError_t* err);

}  // namespace fsr
