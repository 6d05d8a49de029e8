// Spatial hashing that allocates nothing (fsr_spatial_hash_noalloc).
//
// The same hashing as a reconstruct frame (cell key, stable radix sort,
// cell ranges, sorted particle gather), but every scratch buffer lives in
// one file-scope __device__ array instead of memory obtained from
// cudaMalloc.  The caller passes its input and output buffers.
//
// The array is a module global: every process that loads the library holds
// FSR_NOALLOC_MAX_PARTICLES-sized scratch on each device it touches until
// the process exits; all calls on a device share it.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fsr.h"
#include "fsr_internal.h"
#include "kernels.h"
#include "primitives.h"

namespace fsr {
namespace {

constexpr uint32_t kMax = FSR_NOALLOC_MAX_PARTICLES;
// radix_scratch_words(kMax): 4096-element tiles x 256 digits of histogram
// plus the scan's tile sums
constexpr size_t kRadixTiles = (kMax + 4095) / 4096;
constexpr size_t kRadixWords = kRadixTiles * 256 + (kRadixTiles * 256 + 4095) / 4096 + 2;
constexpr size_t kCounterWords = sizeof(Counters) / 4;
constexpr size_t kScratchWords = 4 * (size_t)kMax + kRadixWords + kCounterWords;

// keys0 | vals0 | keys1 | vals1 | radix scratch | Counters
static __device__ __align__(256) uint32_t g_hash_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t* g_scratch_addr[kMaxDevices] = {};

// Device address of g_hash_scratch on the current device.  In host code the
// symbol itself is only a host-side stand-in, never a device address.
cudaError_t scratch_address(uint32_t** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_hash_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

__global__ void k_gather_split(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm, uint32_t n,
                               const float* __restrict__ xyz, const float* __restrict__ dens,
                               float* __restrict__ out_xyz, float* __restrict__ out_den,
                               uint32_t* __restrict__ ranges, uint32_t* __restrict__ out_perm)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = skeys[k];
    if (k == 0 || skeys[k - 1] != key) ranges[2ull * key] = k;
    if (k + 1 == n || skeys[k + 1] != key) ranges[2ull * key + 1] = k + 1;
    const uint32_t s = perm[k];
    out_xyz[3ull * k] = xyz[3ull * s];
    out_xyz[3ull * k + 1] = xyz[3ull * s + 1];
    out_xyz[3ull * k + 2] = xyz[3ull * s + 2];
    out_den[k] = dens[s];
    if (out_perm) out_perm[k] = s;
}

__global__ void k_copy_flag(const Counters* ctr, uint32_t* out) { *out = ctr->out_of_grid; }

}  // namespace
}  // namespace fsr

extern "C" fsr_status fsr_spatial_hash_noalloc(const fsr_frame_header* hdr, float cell_size_scale,
                                               const float* d_xyz, const float* d_density, uint32_t n,
                                               float* d_sorted_xyz, float* d_sorted_density,
                                               uint32_t* d_cell_ranges, uint64_t cell_capacity,
                                               uint32_t* d_perm, uint32_t* d_out_of_grid,
                                               uint64_t* n_cells, void* stream)
{
    using namespace fsr;
    if (!hdr || !n_cells) return FSR_ERR_INVALID_ARGUMENT;
    // an error left pending by earlier work on this thread is not this
    // call's: report it without consuming it, and queue nothing
    if (cudaPeekAtLastError() != cudaSuccess) return FSR_ERR_CUDA;
    if (n > kMax) return FSR_ERR_TOO_LARGE;  // beyond the static scratch
    if (n > 0 && (!d_xyz || !d_density || !d_sorted_xyz || !d_sorted_density)) return FSR_ERR_INVALID_ARGUMENT;
    fsr_params p{};
    p.cell_size_scale = cell_size_scale;
    p.grid_ratio = 1;
    Grid sp{}, sc{};
    uint64_t C = 0, V = 0;
    if (!(hdr->kernel_radius > 0.0f) || !derive_grids(*hdr, p, sp, sc, nullptr, C, V))
        return FSR_ERR_INVALID_ARGUMENT;
    if (C >= 0xFFFFFFFFull) return FSR_ERR_TOO_LARGE;
    *n_cells = C;
    if (!d_cell_ranges || cell_capacity < C) return FSR_ERR_CAPACITY;

    uint32_t* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return FSR_ERR_CUDA;
    uint32_t* k0 = base;
    uint32_t* v0 = k0 + kMax;
    uint32_t* k1 = v0 + kMax;
    uint32_t* v1 = k1 + kMax;
    uint32_t* radix = v1 + kMax;
    Counters* ctr = reinterpret_cast<Counters*>(radix + kRadixWords);

    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const KernelCtx kc{st, sms};
    // the scratch keeps the previous call's contents: clear the counters
    if (cudaMemsetAsync(ctr, 0, sizeof(Counters), st) != cudaSuccess) return FSR_ERR_CUDA;
    if (cudaMemsetAsync(d_cell_ranges, 0xFF, 8ull * C, st) != cudaSuccess) return FSR_ERR_CUDA;
    if (n > 0) {
        launch_hash(kc, d_xyz, n, sp, k0, v0, ctr);
        cudaError_t se = cudaSuccess;
        const int which = radix_sort_pairs(k0, v0, k1, v1, n, bits_for(C), radix, st, &se);
        if (se != cudaSuccess) return FSR_ERR_CUDA;
        const uint32_t* skeys = which ? k1 : k0;
        const uint32_t* perm = which ? v1 : v0;
        k_gather_split<<<(n + 255) / 256, 256, 0, st>>>(skeys, perm, n, d_xyz, d_density, d_sorted_xyz,
                                                        d_sorted_density, d_cell_ranges, d_perm);
    }
    if (d_out_of_grid) k_copy_flag<<<1, 1, 0, st>>>(ctr, d_out_of_grid);
    return cudaGetLastError() == cudaSuccess ? FSR_OK : FSR_ERR_CUDA;
}
