// Vertex welding: the triangle soup of generateTriangles (three unshared
// vertices per triangle, ReconstructionCUDA.cu:451-462) as an indexed mesh.
//
// Every soup vertex lies on one edge of the scalar grid; k_mc_generate
// writes that edge's key, 3 x (linear id of its lower end point) + axis.
// Soup vertices with the same key are the same surface point (computed by
// the cubes that share the edge) and become one mesh vertex:
//   1. insert: a hash table (open addressing, at least twice the soup's
//      capacity, so at most half full) maps each key to a slot; the slot
//      keeps the smallest soup index that carries the key (its first
//      occurrence);
//   2. scan: the first occurrences, in soup order, are numbered 0, 1, ...;
//   3. emit: each soup vertex gets its first occurrence's number as its
//      index; first occurrences copy their position and normal.
// The welded vertices come in order of first use and take the position and
// normal of their first occurrence, so the result does not depend on thread
// scheduling.  All sizes are read on the device (no host round trip).
#include <algorithm>

#include "kernels.h"
#include "primitives.h"

namespace fsr {
namespace {

constexpr uint64_t kEmptyKey = ~0ull;

__device__ __forceinline__ uint32_t hash_slot(uint64_t key, uint32_t shift)
{
    return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> shift);  // Fibonacci hashing
}

__device__ __forceinline__ uint32_t soup_count(const Counters* ctr, uint32_t cap)
{
    const uint32_t n = ctr->n_mesh_verts;
    return n > cap ? 0u : n;  // an overflowing frame is re-run; nothing to weld
}

__global__ void k_weld_insert(WeldArgs a, const Counters* ctr)
{
    const uint32_t n = soup_count(ctr, a.cap);
    const uint32_t mask = a.table_size - 1u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t key = a.keys[i];
        uint32_t s = hash_slot(key, a.shift);
        // at most half the table is in use, so a free slot or the key is
        // found well before the probe count reaches the table size
        for (uint32_t probe = 0; probe < a.table_size; ++probe) {
            const unsigned long long prev =
                atomicCAS(reinterpret_cast<unsigned long long*>(a.table_keys) + s, kEmptyKey, key);
            if (prev == kEmptyKey || prev == key) {
                atomicMin(a.table_first + s, i);
                a.slot[i] = s;
                break;
            }
            s = (s + 1u) & mask;
        }
    }
}

__global__ void k_weld_first(WeldArgs a, const Counters* ctr)
{
    const uint32_t n = soup_count(ctr, a.cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        a.rank[i] = a.table_first[a.slot[i]] == i ? 1u : 0u;
}

__global__ void k_weld_emit(WeldArgs a, const Counters* ctr)
{
    const uint32_t n = soup_count(ctr, a.cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t first = a.table_first[a.slot[i]];
        const uint32_t id = a.rank[first];
        a.index[i] = id;
        if (first == i) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                a.out_pos[3ull * id + k] = a.pos[3ull * i + k];
                a.out_nrm[3ull * id + k] = a.nrm[3ull * i + k];
            }
        }
    }
}

}  // namespace

uint32_t weld_table_size(uint32_t cap)
{
    uint32_t t = 64;
    while (t < 2ull * cap && t < (1u << 31)) t <<= 1;
    return t;
}

cudaError_t launch_weld(const KernelCtx& c, WeldArgs a, Counters* ctr, uint32_t* scan_scratch)
{
    uint32_t lg = 0;
    while ((1u << lg) < a.table_size) ++lg;
    a.shift = 64u - lg;
    cudaError_t e = cudaMemsetAsync(a.table_keys, 0xFF, 8ull * a.table_size, c.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.table_first, 0xFF, 4ull * a.table_size, c.stream);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)std::max(1, c.num_sms * 8);
    k_weld_insert<<<grid, 256, 0, c.stream>>>(a, ctr);
    k_weld_first<<<grid, 256, 0, c.stream>>>(a, ctr);
    // numbers of the first occurrences (in place); the count lands in n_weld
    e = scan_u32(a.rank, a.rank, 0, &ctr->n_mesh_verts, a.cap, &ctr->n_weld, ScanInput::kValue, scan_scratch,
                 c.stream);
    if (e != cudaSuccess) return e;
    k_weld_emit<<<grid, 256, 0, c.stream>>>(a, ctr);
    g_launches += 3;
    return cudaGetLastError();
}

}  // namespace fsr
