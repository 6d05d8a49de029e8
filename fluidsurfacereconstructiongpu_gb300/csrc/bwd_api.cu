// fsr_backward and fsr_copy_mesh_device (include/fsr.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "../../include/fsr.h"
#include "backward.h"
#include "fsr_internal.h"

using namespace fsr;

namespace {

fsr_status bwd_fail(fsr_handle* h, fsr_status s, const std::string& msg)
{
    h->last_error = msg;
    return s;
}

#define BCK(call)                                                                                        \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return bwd_fail(h, e_ == cudaErrorMemoryAllocation ? FSR_ERR_OUT_OF_MEMORY : FSR_ERR_CUDA,   \
                            std::string(#call ": ") + cudaGetErrorString(e_));                           \
    } while (0)

}  // namespace

extern "C" fsr_status fsr_copy_mesh_device(fsr_handle* h, float* d_pos, float* d_nrm, uint64_t capacity,
                                           uint64_t* n_vertices, void* stream)
{
    if (!h || !n_vertices) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return bwd_fail(h, FSR_ERR_NOT_READY, "no frame reconstructed");
    const uint64_t nv = h->stats.n_mesh_vertices;
    *n_vertices = nv;
    if (nv > capacity) return bwd_fail(h, FSR_ERR_CAPACITY, "mesh buffer too small");
    if (nv == 0) return FSR_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (d_pos) BCK(cudaMemcpyAsync(d_pos, h->mesh_pos.ptr, 12ull * nv, cudaMemcpyDeviceToDevice, st));
    if (d_nrm) BCK(cudaMemcpyAsync(d_nrm, h->mesh_nrm.ptr, 12ull * nv, cudaMemcpyDeviceToDevice, st));
    return FSR_OK;
}

extern "C" fsr_status fsr_backward(fsr_handle* h, const float* d_grad_mesh_pos, float* d_grad_xyz,
                                   float* grad_particle_radius, void* stream)
{
    if (!h) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return bwd_fail(h, FSR_ERR_NOT_READY, "no frame reconstructed");
    if (h->params.flags & FSR_FLAG_COMPUTE_DENSITY)
        return bwd_fail(h, FSR_ERR_INVALID_ARGUMENT, "no backward pass for frames with computed densities");
    const uint64_t n = h->n_last;
    if (n > 0 && !d_grad_xyz) return bwd_fail(h, FSR_ERR_INVALID_ARGUMENT, "null gradient output");
    if (h->stats.n_mesh_vertices > 0 && !d_grad_mesh_pos)
        return bwd_fail(h, FSR_ERR_INVALID_ARGUMENT, "null mesh gradient");
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != h->device) cudaSetDevice(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    const fsr_params& p = h->params;
    const Grid sp = h->grid_sp, sc = h->grid_sc;
    const uint64_t keys = (uint64_t)(sp.res[0] + 1) * (sp.res[1] + 1) * (sp.res[2] + 1);
    const uint64_t nn = std::max<uint64_t>(n, 1);
    BCK(h->gphi.ensure(4ull * h->cap_band));
    BCK(h->gkey.ensure(4ull * keys));
    BCK(h->gklist.ensure(4ull * (keys + 4)));
    BCK(h->gx.ensure(16ull * nn));
    BCK(h->gscalar.ensure(16));
    if (p.method == FSR_METHOD_YU13) {
        BCK(h->gsmooth.ensure(16ull * nn));
        BCK(h->gG.ensure(48ull * nn));
        BCK(h->gmean.ensure(16ull * nn));
    }
    if (!h->tri.ptr) {
        BCK(h->tri.ensure(sizeof(mc::kTriPacked)));
        BCK(cudaMemcpy(h->tri.ptr, mc::kTriPacked, sizeof(mc::kTriPacked), cudaMemcpyHostToDevice));
    }
    BCK(cudaMemsetAsync(h->gphi.ptr, 0, 4ull * h->cap_band, st));
    BCK(cudaMemsetAsync(h->gkey.ptr, 0, 4ull * keys, st));
    BCK(cudaMemsetAsync(h->gklist.ptr, 0, 16, st));
    BCK(cudaMemsetAsync(h->gx.ptr, 0, 16ull * nn, st));
    BCK(cudaMemsetAsync(h->gscalar.ptr, 0, 16, st));
    if (p.method == FSR_METHOD_YU13) {
        BCK(cudaMemsetAsync(h->gsmooth.ptr, 0, 16ull * nn, st));
        BCK(cudaMemsetAsync(h->gG.ptr, 0, 48ull * nn, st));
    }

    BwdArgs a{};
    a.sp = sp;
    a.sc = sc;
    a.ratio = p.grid_ratio;
    a.n = (uint32_t)n;
    a.band = BandView{(const uint32_t*)h->bits.ptr, (const uint32_t*)h->prefix.ptr, (const float*)h->phi.ptr};
    a.sv = (const uint32_t*)h->sv.ptr;
    a.valid = (const uint32_t*)h->valid.ptr;
    a.mc = (const uint32_t*)h->mc.ptr;
    a.vofs = (const uint32_t*)h->vofs.ptr;
    a.tri = (const uint64_t*)h->tri.ptr;
    a.gmesh = d_grad_mesh_pos;
    a.gphi = (float*)h->gphi.ptr;
    a.gkey = (uint32_t*)h->gkey.ptr;
    a.glist = (uint32_t*)h->gklist.ptr;
    a.sorted = (const float4*)h->sorted.ptr;
    a.skeys = h->skeys_ptr;
    a.perm = h->perm_ptr;
    a.invol = (const uint8_t*)h->invol.ptr;
    a.smoothed = (const float4*)h->smoothed.ptr;
    a.grec = (const float4*)h->grec.ptr;
    a.qrec = (const float4*)h->qrec.ptr;
    a.ranges = (const uint2*)h->ranges.ptr;
    a.cell_rmax = (const float*)h->cell_rmax.ptr;
    a.mv = (const float4*)h->mv.ptr;
    a.gsmooth = (float4*)h->gsmooth.ptr;
    a.gG = (float4*)h->gG.ptr;
    a.gmean = (float4*)h->gmean.ptr;
    a.gx = (float4*)h->gx.ptr;
    a.iso = p.iso_value;
    a.h = h->hdr_last.kernel_radius;
    a.sigma = 315.0f / (64.0f * 3.1415926535898f);
    a.cap_band = h->cap_band;
    a.cap_valid = h->cap_valid;

    CovArgs ca{};
    const float R = h->hdr_last.kernel_radius * p.aniso_radius_over_h;
    if (p.method == FSR_METHOD_YU13) {
        ca.sp = sp;
        ca.sorted = (const float4*)h->sorted.ptr;
        ca.mean = (const float4*)h->mean.ptr;
        ca.mean32 = (const float4*)h->mean32.ptr;
        ca.smoothed = (const float4*)h->smoothed.ptr;
        ca.crec = (float4*)h->covrec.ptr;
        ca.ranges = (const uint2*)h->ranges.ptr;
        ca.skeys = h->skeys_ptr;
        ca.invol = (const uint8_t*)h->invol.ptr;
        ca.n = (uint32_t)n;
        ca.R = R;
        ca.h = h->hdr_last.kernel_radius;
        ca.h2 = ca.h * ca.h;
        ca.h_inv = (float)(1.0 / (double)ca.h);
        ca.mass = h->hdr_last.particle_mass;
        ca.sigma = a.sigma;
        ca.min_neighbors = p.min_neighbors;
        ca.R_lt2 = sqrt_threshold(R, false);
        ca.R_le2 = sqrt_threshold(R, true);
        // as in the forward: compact warps may walk the union of their windows
        ca.coop_ok = (R + R * 1.0001f + 1e-4f * sp.cs) < 2.0f * sp.cs * 0.9999f ? 1 : 0;
    }
    const KernelCtx kc{st, h->num_sms};
    const bool want_radius = grad_particle_radius && (p.method == FSR_METHOD_ZB05 || p.method == FSR_METHOD_AKINCI12);
    const uint64_t launches0 = g_launches;
    if (n > 0)
        launch_backward(kc, a, &ca, (const Counters*)h->ctr.ptr, (int)p.method, p.smoothing_lambda, R,
                        want_radius ? (float*)h->gscalar.ptr : nullptr, d_grad_xyz);
    BCK(cudaGetLastError());
    h->stats.n_backward_launches = (uint32_t)(g_launches - launches0);
    h->stats.device_bytes = 0;
    for (DevBuf* b : h->all_buffers()) h->stats.device_bytes += b->bytes;
    if (grad_particle_radius) {
        float r = 0.f;
        if (want_radius) {
            BCK(cudaMemcpyAsync(&r, h->gscalar.ptr, 4, cudaMemcpyDeviceToHost, st));
            BCK(cudaStreamSynchronize(st));
        }
        *grad_particle_radius = r;
    }
    if (prev != h->device) cudaSetDevice(prev);
    return FSR_OK;
}
