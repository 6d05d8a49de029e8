// Pair counts of the last frame's neighbour-sum stages (fsr_count_pairs).
//
// A diagnostic for throughput accounting, with no counterpart in the
// reference.  For every neighbour-sum stage it counts, by brute force over
// the frame's kept buffers, the candidate pairs the reference's loops visit
// (every particle of the unit's cell window) and the pairs inside the
// kernel's support, which are the ones that add non-zero terms:
//   smoothing  particles x +-2 cells, d < R              (cu:598-658)
//   covariance involved particles x +-2 cells, |x - mean| < R (cu:689-827)
//   aniso field band vertices x +-2 cells, |G (x~ - v)| < 1 for involved
//              particles and |x~ - v| < 1 for the others  (cu:830-906)
//   ZB05/TC01  band vertices x +-1 cells, d < h          (cu:178-289)
//   colour     particles x +-1 cells, 0 < d < h          (cu:909-971)
// One thread per unit walks its window the way the reference does; the
// counts are reduced per warp into 64-bit counters.
#include <cuda_runtime.h>

#include "../../include/fsr.h"
#include "fsr_internal.h"

namespace fsr {
namespace {

struct PairCtr {
    unsigned long long cand, contrib;
};

__device__ __forceinline__ void warp_add(PairCtr* c, uint64_t cand, uint64_t contrib)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_xor_sync(0xffffffffu, cand, o);
        contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
    }
    if ((threadIdx.x & 31) == 0 && cand) {
        atomicAdd(&c->cand, (unsigned long long)cand);
        atomicAdd(&c->contrib, (unsigned long long)contrib);
    }
}

// Particles (smoothing, colour field; covariance when `mean` is given, over
// involved particles only): ext-cell windows about the particle's cell, the
// support test about the particle (or its mean).
__global__ void k_count_particles(const float4* __restrict__ sorted, uint32_t n, const uint2* __restrict__ ranges,
                                  Grid sp, int ext, float r2, bool skip_self_zero, const float4* __restrict__ mean,
                                  const uint8_t* __restrict__ invol, const uint32_t* __restrict__ skeys, PairCtr* out)
{
    uint64_t cand = 0, contrib = 0;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t - threadIdx.x < n; t += gridDim.x * blockDim.x) {
        if (t < n && !(invol && !invol[skeys[t]])) {
            const float4 p = sorted[t];
            const float4 c = mean ? mean[t] : p;
            const Window w = window(cell1(p.x, sp.min[0], sp.cs), cell1(p.y, sp.min[1], sp.cs),
                                    cell1(p.z, sp.min[2], sp.cs), ext, sp);
            for (int z = w.lo[2]; z <= w.hi[2]; ++z)
                for (int y = w.lo[1]; y <= w.hi[1]; ++y)
                    for (int x = w.lo[0]; x <= w.hi[0]; ++x) {
                        const uint2 r = ranges[lin3(x, y, z, sp)];
                        if (r.x == kEmpty) continue;
                        cand += r.y - r.x;
                        for (uint32_t i = r.x; i < r.y; ++i) {
                            const float4 q = __ldg(&sorted[i]);
                            const float dx = q.x - c.x, dy = q.y - c.y, dz = q.z - c.z;
                            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            contrib += (d2 < r2 && !(skip_self_zero && d2 == 0.f)) ? 1u : 0u;
                        }
                    }
        }
        warp_add(out, cand, contrib);
        cand = contrib = 0;
    }
}

// Band vertices: ext-cell windows about the vertex's cell.  aniso: the
// involved particles' records (x~, r2max) (M00, 2M01, 2M02, coef)
// (M11, 2M12, M22, 0) with M = G^T G, the smoothed positions of the others;
// otherwise d < sqrt(r2) about the sorted positions.
__global__ void k_count_vertices(const uint32_t* __restrict__ sv, uint32_t nb, Grid sc, Grid sp,
                                 const uint2* __restrict__ ranges, int ext, float r2,
                                 const float4* __restrict__ sorted, const float4* __restrict__ qrec,
                                 const float4* __restrict__ smoothed, const uint8_t* __restrict__ invol,
                                 PairCtr* out)
{
    uint64_t cand = 0, contrib = 0;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t - threadIdx.x < nb; t += gridDim.x * blockDim.x) {
        if (t < nb) {
            uint32_t vx, vy, vz;
            unlin3(sv[t], sc, vx, vy, vz);
            const float px = vpos1(vx, sc.min[0], sc.cs), py = vpos1(vy, sc.min[1], sc.cs),
                        pz = vpos1(vz, sc.min[2], sc.cs);
            const Window w = window(cell1(px, sp.min[0], sp.cs), cell1(py, sp.min[1], sp.cs),
                                    cell1(pz, sp.min[2], sp.cs), ext, sp);
            for (int z = w.lo[2]; z <= w.hi[2]; ++z)
                for (int y = w.lo[1]; y <= w.hi[1]; ++y)
                    for (int x = w.lo[0]; x <= w.hi[0]; ++x) {
                        const uint32_t cell = lin3(x, y, z, sp);
                        const uint2 r = ranges[cell];
                        if (r.x == kEmpty) continue;
                        cand += r.y - r.x;
                        const bool inv = qrec && invol[cell];
                        for (uint32_t i = r.x; i < r.y; ++i) {
                            if (qrec && inv) {
                                const float4 a = __ldg(&qrec[3ull * i]), b = __ldg(&qrec[3ull * i + 1]),
                                             c = __ldg(&qrec[3ull * i + 2]);
                                const float dx = a.x - px, dy = a.y - py, dz = a.z - pz;
                                const float q2 = fmaf(b.x * dx, dx, fmaf(b.y * dx, dy, fmaf(b.z * dx, dz,
                                                 fmaf(c.x * dy, dy, fmaf(c.y * dy, dz, c.z * dz * dz)))));
                                contrib += q2 < 1.0f ? 1u : 0u;
                            } else {
                                const float4 q = qrec ? __ldg(&smoothed[i]) : __ldg(&sorted[i]);
                                const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
                                contrib += fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < r2 ? 1u : 0u;
                            }
                        }
                    }
        }
        warp_add(out, cand, contrib);
        cand = contrib = 0;
    }
}

unsigned grid_for(uint64_t n, int sms)
{
    const uint64_t want = (n + 255) / 256;
    const uint64_t most = (uint64_t)sms * 8;
    return (unsigned)(want < 1 ? 1 : (want > most ? most : want));
}

}  // namespace
}  // namespace fsr

extern "C" fsr_status fsr_count_pairs(fsr_handle* h, fsr_pair_counts* out, void* stream)
{
    using namespace fsr;
    if (!h || !out) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) {
        h->last_error = "fsr_count_pairs: no frame";
        return FSR_ERR_NOT_READY;
    }
    *out = fsr_pair_counts{};
    if (cudaSetDevice(h->device) != cudaSuccess) return FSR_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    const fsr_params& p = h->params;
    const uint32_t n = (uint32_t)h->n_last;
    const uint32_t nb = (uint32_t)h->stats.n_band_vertices;
    const Grid sp = h->grid_sp, sc = h->grid_sc;
    const float hr = h->hdr_last.kernel_radius;
    const float4* sorted = (const float4*)h->sorted.ptr;
    const uint2* ranges = (const uint2*)h->ranges.ptr;
    PairCtr* d = nullptr;
    if (cudaMallocAsync((void**)&d, 4 * sizeof(PairCtr), st) != cudaSuccess) return FSR_ERR_CUDA;
    cudaMemsetAsync(d, 0, 4 * sizeof(PairCtr), st);
    const int sms = h->num_sms;
    const bool yu13 = p.method == FSR_METHOD_YU13;
    if (n && yu13) {
        const float R = hr * p.aniso_radius_over_h;
        k_count_particles<<<grid_for(n, sms), 256, 0, st>>>(sorted, n, ranges, sp, 2, R * R, false, nullptr,
                                                           nullptr, nullptr, d + 0);
        k_count_particles<<<grid_for(n, sms), 256, 0, st>>>(sorted, n, ranges, sp, 2, R * R, false,
                                                           (const float4*)h->mean.ptr,
                                                           (const uint8_t*)h->invol.ptr, h->skeys_ptr, d + 1);
    }
    if (n && p.method == FSR_METHOD_AKINCI12)
        k_count_particles<<<grid_for(n, sms), 256, 0, st>>>(sorted, n, ranges, sp, 1, hr * hr, true, nullptr,
                                                           nullptr, nullptr, d + 3);
    if (nb) {
        if (yu13)
            k_count_vertices<<<grid_for(nb, sms), 256, 0, st>>>(
                (const uint32_t*)h->sv.ptr, nb, sc, sp, ranges, 2, 1.0f, sorted, (const float4*)h->qrec.ptr,
                (const float4*)h->smoothed.ptr, (const uint8_t*)h->invol.ptr, d + 2);
        else
            k_count_vertices<<<grid_for(nb, sms), 256, 0, st>>>((const uint32_t*)h->sv.ptr, nb, sc, sp, ranges, 1,
                                                               hr * hr, sorted, nullptr, nullptr, nullptr, d + 2);
    }
    PairCtr hc[4] = {};
    cudaError_t e = cudaMemcpyAsync(hc, d, sizeof(hc), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(d, st);
    if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return FSR_ERR_CUDA;
    out->smooth_candidates = hc[0].cand;
    out->smooth_contributing = hc[0].contrib;
    out->cov_candidates = hc[1].cand;
    out->cov_contributing = hc[1].contrib;
    out->field_candidates = hc[2].cand;
    out->field_contributing = hc[2].contrib;
    out->color_candidates = hc[3].cand;
    out->color_contributing = hc[3].contrib;
    return FSR_OK;
}
