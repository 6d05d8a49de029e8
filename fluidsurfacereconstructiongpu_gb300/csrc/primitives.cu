// Exclusive scan (reduce-then-scan over 4096-element tiles) and stable LSD
// radix sort (8-bit digits, per-warp match-based ranking).
#include "primitives.h"
#include "kernels.h"

#include <algorithm>

namespace fsr {
namespace {

template <ScanInput M>
__device__ __forceinline__ uint32_t scan_load(const uint32_t* in, uint32_t i)
{
    const uint32_t v = __ldg(in + i);
    if (M == ScanInput::kPopcount) return __popc(v);
    if (M == ScanInput::kNonzero) return v != 0u ? 1u : 0u;
    return v;
}

__device__ __forceinline__ uint32_t count_of(uint32_t n_host, const uint32_t* n_dev, uint32_t n_max)
{
    const uint32_t n = n_dev ? *n_dev : n_host;
    return n < n_max ? n : n_max;
}

template <ScanInput M>
__global__ void __launch_bounds__(kScanThreads) k_tile_reduce(const uint32_t* in, uint32_t n_host,
                                                              const uint32_t* n_dev, uint32_t n_max,
                                                              uint32_t* tile_sums)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t n = count_of(n_host, n_dev, n_max);
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t base = (uint64_t)tile * kScanTile;
        uint32_t s = 0;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint64_t i = base + k * kScanThreads + threadIdx.x;
            if (i < n) s += scan_load<M>(in, (uint32_t)i);
        }
        const uint32_t incl = block_inclusive_scan(s, warp_sums);
        if (threadIdx.x == kScanThreads - 1) tile_sums[tile] = incl;
        __syncthreads();
    }
}

// Single block: exclusive scan of the tile sums in place; total to *total.
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(uint32_t* tile_sums, uint32_t n_host,
                                                                 const uint32_t* n_dev, uint32_t n_max,
                                                                 uint32_t* total)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t n = count_of(n_host, n_dev, n_max);
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    uint32_t carry = 0;
    for (uint32_t b = 0; b < ntiles; b += kScanThreads) {
        const uint32_t i = b + threadIdx.x;
        const uint32_t x = i < ntiles ? tile_sums[i] : 0u;
        const uint32_t incl = block_inclusive_scan(x, warp_sums);
        if (i < ntiles) tile_sums[i] = carry + incl - x;
        __shared__ uint32_t last;
        if (threadIdx.x == kScanThreads - 1) last = incl;
        __syncthreads();
        carry += last;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

template <ScanInput M>
__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const uint32_t* in, uint32_t* out,
                                                            uint32_t n_host, const uint32_t* n_dev,
                                                            uint32_t n_max, const uint32_t* tile_prefix)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    __shared__ uint32_t tile_vals[kScanTile];
    const uint32_t n = count_of(n_host, n_dev, n_max);
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t base = (uint64_t)tile * kScanTile;
        // coalesced load into shared memory
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t j = k * kScanThreads + threadIdx.x;
            const uint64_t i = base + j;
            tile_vals[j] = i < n ? scan_load<M>(in, (uint32_t)i) : 0u;
        }
        __syncthreads();
        // each thread owns kScanItems consecutive elements
        uint32_t local[kScanItems];
        uint32_t s = 0;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            local[k] = tile_vals[threadIdx.x * kScanItems + k];
            s += local[k];
        }
        const uint32_t incl = block_inclusive_scan(s, warp_sums);
        uint32_t run = tile_prefix[tile] + incl - s;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            tile_vals[threadIdx.x * kScanItems + k] = run;
            run += local[k];
        }
        __syncthreads();
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t j = k * kScanThreads + threadIdx.x;
            const uint64_t i = base + j;
            if (i < n) out[i] = tile_vals[j];
        }
        __syncthreads();
    }
}

template <ScanInput M>
void launch_scan(uint32_t g, const uint32_t* in, uint32_t* out, uint32_t n_host, const uint32_t* n_dev,
                 uint32_t n_max, uint32_t* total, uint32_t* scratch, cudaStream_t stream)
{
    k_tile_reduce<M><<<g, kScanThreads, 0, stream>>>(in, n_host, n_dev, n_max, scratch);
    k_scan_tile_sums<<<1, kScanThreads, 0, stream>>>(scratch, n_host, n_dev, n_max, total);
    k_tile_scan<M><<<g, kScanThreads, 0, stream>>>(in, out, n_host, n_dev, n_max, scratch);
    g_launches += 3;
}

uint32_t grid_for_tiles(uint64_t n_max)
{
    const uint64_t t = (n_max + kScanTile - 1) / kScanTile;
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(t, 65535));
}

// One-block exclusive scan (in place allowed) for short arrays: tiles of
// 4 x 1024 consecutive elements, each thread four of them, a block scan per
// tile and a running carry.  One launch instead of three.
constexpr uint32_t kSingleThreads = 1024;
constexpr uint32_t kSingleMax = 1u << 14;  // longer arrays take the tiled three-kernel scan (one block is slower from ~64k on)
__global__ void __launch_bounds__(kSingleThreads) k_scan_single(const uint32_t* in, uint32_t* out, uint32_t n)
{
    __shared__ uint32_t warp_sums[kSingleThreads / 32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < n; base += 4 * kSingleThreads) {
        const uint32_t i0 = base + 4 * threadIdx.x;
        uint32_t v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = i0 + k < n ? in[i0 + k] : 0u;
        const uint32_t s = v[0] + v[1] + v[2] + v[3];
        uint32_t x = s;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sums[lane];
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        uint32_t run = carry + x - s + (warp ? warp_sums[warp - 1] : 0u);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i0 + k < n) out[i0 + k] = run;
            run += v[k];
        }
        carry += warp_sums[kSingleThreads / 32 - 1];
        __syncthreads();  // warp_sums is rewritten by the next tile
    }
}

// ---------------------------------------------------------------- radix

constexpr uint32_t kRadixBits = 8;
constexpr uint32_t kRadixBins = 1u << kRadixBits;
constexpr uint32_t kRadixThreads = 256;
constexpr uint32_t kRadixItems = 16;
constexpr uint32_t kRadixTile = kRadixThreads * kRadixItems;  // 4096
constexpr uint32_t kRadixWarps = kRadixThreads / 32;

__global__ void __launch_bounds__(kRadixThreads) k_radix_hist(const uint32_t* keys, uint32_t n,
                                                              uint32_t shift, uint32_t ntiles,
                                                              uint32_t* hist)
{
    __shared__ uint32_t h[kRadixBins];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kRadixTile;
#pragma unroll 4
    for (uint32_t k = 0; k < kRadixItems; ++k) {
        const uint64_t i = base + k * kRadixThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(__ldg(keys + i) >> shift) & (kRadixBins - 1)], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter.  Warp w owns the tile's elements [w*512, (w+1)*512) and
// walks them in 16 rounds of 32 consecutive elements, so (warp, round, lane)
// is memory order; ranks within a warp come from __match_any_sync and a
// per-warp digit counter, ranks across warps from an exclusive scan of those
// counters.
__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(const uint32_t* kin, const uint32_t* vin,
                                                                 uint32_t* kout, uint32_t* vout, uint32_t n,
                                                                 uint32_t shift, uint32_t ntiles,
                                                                 const uint32_t* offsets)
{
    __shared__ uint32_t whist[kRadixWarps][kRadixBins];
    __shared__ uint32_t base[kRadixBins];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t w = 0; w < kRadixWarps; ++w) whist[w][threadIdx.x] = 0;
    base[threadIdx.x] = offsets[threadIdx.x * ntiles + blockIdx.x];
    __syncthreads();

    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint64_t wbase = (uint64_t)blockIdx.x * kRadixTile + (uint64_t)warp * (32u * kRadixItems);
    uint32_t kk[kRadixItems], vv[kRadixItems], rr[kRadixItems];
#pragma unroll
    for (uint32_t r = 0; r < kRadixItems; ++r) {
        const uint64_t i = wbase + r * 32u + lane;
        const bool ok = i < n;
        const uint32_t key = ok ? __ldg(kin + i) : 0u;
        const uint32_t d = (key >> shift) & (kRadixBins - 1);
        const uint32_t peers = __match_any_sync(0xffffffffu, ok ? d : 0x100u);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (ok && lane == leader) {
            before = whist[warp][d];
            whist[warp][d] = before + __popc(peers);
        }
        before = __shfl_sync(0xffffffffu, before, leader);
        __syncwarp();
        kk[r] = key;
        vv[r] = ok ? __ldg(vin + i) : 0u;
        rr[r] = before + __popc(peers & lt_mask);
    }
    __syncthreads();
    {
        uint32_t run = 0;
        for (uint32_t w = 0; w < kRadixWarps; ++w) {
            const uint32_t c = whist[w][threadIdx.x];
            whist[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (uint32_t r = 0; r < kRadixItems; ++r) {
        const uint64_t i = wbase + r * 32u + lane;
        if (i < n) {
            const uint32_t d = (kk[r] >> shift) & (kRadixBins - 1);
            const uint32_t pos = base[d] + whist[warp][d] + rr[r];
            kout[pos] = kk[r];
            vout[pos] = vv[r];
        }
    }
}

}  // namespace

size_t scan_scratch_words(uint64_t n_max)
{
    return (size_t)((n_max + kScanTile - 1) / kScanTile) + 1;
}

cudaError_t scan_u32(const uint32_t* in, uint32_t* out, uint32_t n_host, const uint32_t* n_dev,
                     uint32_t n_max, uint32_t* total, ScanInput mode, uint32_t* scratch,
                     cudaStream_t stream)
{
    if (n_max == 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), stream);
        return cudaSuccess;
    }
    const uint32_t g = grid_for_tiles(n_max);
    switch (mode) {
    case ScanInput::kValue: launch_scan<ScanInput::kValue>(g, in, out, n_host, n_dev, n_max, total, scratch, stream); break;
    case ScanInput::kPopcount: launch_scan<ScanInput::kPopcount>(g, in, out, n_host, n_dev, n_max, total, scratch, stream); break;
    case ScanInput::kNonzero: launch_scan<ScanInput::kNonzero>(g, in, out, n_host, n_dev, n_max, total, scratch, stream); break;
    }
    return cudaGetLastError();
}

size_t radix_scratch_words(uint32_t n)
{
    const uint64_t ntiles = ((uint64_t)n + kRadixTile - 1) / kRadixTile;
    const uint64_t hist = ntiles * kRadixBins;
    return (size_t)(hist + scan_scratch_words(hist) + 1);
}

int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n,
                     uint32_t key_bits, uint32_t* scratch, cudaStream_t stream, cudaError_t* err)
{
    *err = cudaSuccess;
    if (n <= 1 || key_bits == 0) return 0;
    const uint32_t ntiles = (n + kRadixTile - 1) / kRadixTile;
    const uint32_t nhist = ntiles * kRadixBins;
    uint32_t* hist = scratch;
    uint32_t* scan_tmp = scratch + nhist;
    int cur = 0;
    for (uint32_t shift = 0; shift < key_bits; shift += kRadixBits) {
        const uint32_t* kin = cur ? k1 : k0;
        const uint32_t* vin = cur ? v1 : v0;
        uint32_t* kout = cur ? k0 : k1;
        uint32_t* vout = cur ? v0 : v1;
        k_radix_hist<<<ntiles, kRadixThreads, 0, stream>>>(kin, n, shift, ntiles, hist);
        if (nhist <= kSingleMax) {
            k_scan_single<<<1, kSingleThreads, 0, stream>>>(hist, hist, nhist);
            ++g_launches;
        } else {
            cudaError_t e = scan_u32(hist, hist, nhist, nullptr, nhist, nullptr, ScanInput::kValue, scan_tmp, stream);
            if (e != cudaSuccess) { *err = e; return cur; }
        }
        k_radix_scatter<<<ntiles, kRadixThreads, 0, stream>>>(kin, vin, kout, vout, n, shift, ntiles, hist);
        g_launches += 2;
        cur ^= 1;
    }
    *err = cudaGetLastError();
    return cur;
}

}  // namespace fsr
