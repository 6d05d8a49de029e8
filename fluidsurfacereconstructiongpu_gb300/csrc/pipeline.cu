// Frame orchestration and the fsr_* C ABI (include/fsr.h).
//
// One frame is one queue of kernels on the caller's stream: spatial hashing
// (key + stable radix sort + ranges), surface cells, narrow band (bitset +
// rank directory + band list), field, marching cubes (classify, one scan
// for the vertex offsets and the valid-cube list, generation).  Sizes the reference reads back after every
// scan (ReconstructionCUDA.cu:1164-1171) stay on the device in a Counters
// block; the host reads that block once at the end of the frame.  When a
// pooled buffer turned out too small the frame is re-queued with the grown
// capacities (only the first frames of a new workload pay for that).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fsr.h"
#include "fsr_internal.h"
#include "kernels.h"
#include "primitives.h"

namespace fsr {

// ------------------------------------------------------------ grid derivation
// ReconstructorGPU.cpp:237-268 (spatial grid: bbox grown by one cell,
// res = uint((max - min) / cs + 1) in FP32) and :99-105 (scalar grid: cell
// cs / ratio over the same box).
bool derive_grids(const fsr_frame_header& hdr, const fsr_params& p, Grid& sp, Grid& sc, float* sp_max,
                  uint64_t& C, uint64_t& V)
{
    const volatile float h = hdr.kernel_radius;  // volatile: keep every step in FP32
    const float cs = h * p.cell_size_scale;
    if (!(cs > 0.0f) || p.grid_ratio == 0 || !std::isfinite(cs)) return false;
    const float scs = cs / (float)p.grid_ratio;
    C = 1;
    V = 1;
    for (int a = 0; a < 3; ++a) {
        const volatile float mn = hdr.bbox_min[a] - cs;
        const volatile float mx = hdr.bbox_max[a] + cs;
        const volatile float d = mx - mn;
        const volatile float rs = d / cs + 1.0f;
        const volatile float rv = d / scs + 1.0f;
        if (!(rs >= 1.0f && rs < 4294967296.0f) || !(rv >= 2.0f && rv < 4294967296.0f)) return false;
        sp.min[a] = mn;
        sc.min[a] = mn;
        sp.res[a] = (uint32_t)rs;
        sc.res[a] = (uint32_t)rv;
        if (sp_max) sp_max[a] = mx;
        C *= sp.res[a];
        V *= sc.res[a];
    }
    sp.cs = cs;
    sc.cs = scs;
    sp.pad = sc.pad = 0;
    return true;
}

// Largest float t with (double)t < 1.5 * (double)h: dist <= t <=> the
// reference's `dist < h * 1.5` evaluated in double (cu:587).
float band_threshold(float h)
{
    const double t = (double)h * 1.5;
    float f = (float)t;
    if ((double)f >= t) f = std::nextafterf(f, 0.0f);
    return f;
}

uint32_t bits_for(uint64_t c)
{
    uint32_t b = 0;
    while (b < 32 && (1ull << b) < c) ++b;
    return b;
}

}  // namespace fsr

using namespace fsr;

namespace {

fsr_status fail(fsr_handle* h, fsr_status st, const char* fmt, ...)
{
    if (h) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        h->last_error = buf;
    }
    return st;
}

fsr_status cuda_fail(fsr_handle* h, cudaError_t e, const char* where)
{
    return fail(h, e == cudaErrorMemoryAllocation ? FSR_ERR_OUT_OF_MEMORY : FSR_ERR_CUDA, "%s: %s (%d)", where,
                cudaGetErrorString(e), (int)e);
}

#define CK(call)                                                     \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call);       \
    } while (0)

bool valid_params(const fsr_params& p)
{
    if (p.method > FSR_METHOD_AKINCI12) return false;
    // the field kernels index a group's vertex box with 10 bits per axis (ratio + 1 vertices)
    if (p.grid_ratio == 0 || p.grid_ratio > 1000 || !(p.cell_size_scale > 0.0f) || !std::isfinite(p.iso_value))
        return false;
    if (p.method == FSR_METHOD_YU13 && !(p.aniso_radius_over_h > 0.0f)) return false;
    return true;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

// ------------------------------------------------------------ DevBuf

cudaError_t DevBuf::ensure(size_t want)
{
    if (want <= bytes) return cudaSuccess;
    // the old block may still be read by work queued on another stream (a
    // pipelined sequence uploads and downloads beside the kernels): let the
    // device finish it before the block is freed
    if (ptr) {
        cudaDeviceSynchronize();
        cudaFree(ptr);
    }
    ptr = nullptr;
    bytes = 0;
    const size_t b = std::max<size_t>(want, 256);
    cudaError_t e = cudaMalloc(&ptr, b);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return e;
    }
    bytes = b;
    return cudaSuccess;
}

void DevBuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

fsr_handle::~fsr_handle()
{
    DeviceGuard g(device);
    for (DevBuf* b : all_buffers()) b->release();
    if (pinned_ctr) cudaFreeHost(pinned_ctr);
    if (pinned_ctr_b) cudaFreeHost(pinned_ctr_b);
    for (auto& e : ev) {
        if (e) cudaEventDestroy(e);
    }
    for (int k = 0; k < 2; ++k) {
        if (ev_up[k]) cudaEventDestroy(ev_up[k]);
        if (ev_done[k]) cudaEventDestroy(ev_done[k]);
        if (ev_down[k]) cudaEventDestroy(ev_down[k]);
    }
    if (up) cudaStreamDestroy(up);
    if (down) cudaStreamDestroy(down);
    if (ev_start) cudaEventDestroy(ev_start);
}

std::vector<DevBuf*> fsr_handle::all_buffers()
{
    return {&in_xyz, &in_den,  &keys0,  &vals0,  &keys1, &vals1,  &radix_tmp, &sorted, &ranges,  &occ,
            &surf,   &invol, &cell_rmax,   &psurf,  &bits,   &prefix, &gflag, &glist, &scan_tmp, &sv,       &phi,    &mc,      &vofs,
            &valid,   &mean,   &mean32, &smoothed, &grec, &qrec, &covrec, &mesh_pos, &mesh_nrm, &wkey, &wslot, &wrank, &widx, &wpos, &wnrm, &wtable_keys, &wtable_first, &rho, &pflags, &ctr, &mv, &gphi, &gkey, &gklist, &gsmooth, &gG, &gmean, &gx, &gscalar, &tri, &in_xyz_b, &in_den_b, &mesh_pos_b, &mesh_nrm_b};
}

// ------------------------------------------------------------ frame

namespace fsr {

fsr_status frame_plan(fsr_handle* h, const fsr_frame_header& hdr, uint64_t n64, FramePlan& fp)
{
    const fsr_params& p = h->params;
    if (n64 >= 0xFFFFFFFFull) return fail(h, FSR_ERR_TOO_LARGE, "too many particles: %llu", (unsigned long long)n64);
    if (!(hdr.kernel_radius > 0.0f) || !std::isfinite(hdr.kernel_radius))
        return fail(h, FSR_ERR_INVALID_ARGUMENT, "kernel radius must be positive");
    fp = FramePlan{};
    fp.hdr = hdr;
    fp.n = (uint32_t)n64;
    if (!derive_grids(hdr, p, fp.sp, fp.sc, nullptr, fp.C, fp.V))
        return fail(h, FSR_ERR_INVALID_ARGUMENT, "invalid grid (bounding box, kernel radius or ratio)");
    if (fp.C >= 0xFFFFFFFFull || fp.V >= 0xFFFFFFFFull)
        return fail(h, FSR_ERR_TOO_LARGE, "grid too large: %llu cells, %llu vertices", (unsigned long long)fp.C,
                    (unsigned long long)fp.V);
    fp.nwords = (uint32_t)((fp.V + 31) / 32);
    // capacities of the device-sized arrays
    if (p.flags & FSR_FLAG_SMALL_POOLS) {
        if (h->cap_band == 0) h->cap_band = (uint32_t)std::min<uint64_t>(fp.V, 4096);
        if (h->cap_valid == 0) h->cap_valid = 1024;
        if (h->cap_mesh == 0) h->cap_mesh = 4096;
    }
    if (h->cap_band == 0) h->cap_band = (uint32_t)std::min<uint64_t>(fp.V, std::max<uint64_t>(1u << 20, 24ull * fp.n));
    if (h->cap_valid == 0) h->cap_valid = std::max<uint32_t>(1u << 18, h->cap_band / 4);
    if (h->cap_mesh == 0) h->cap_mesh = std::max<uint32_t>(1u << 20, 4u * h->cap_valid);
    return FSR_OK;
}

fsr_status frame_buffers(fsr_handle* h, const FramePlan& fp)
{
    const fsr_params& p = h->params;
    const bool yu13 = p.method == FSR_METHOD_YU13;
    const bool keep = (p.flags & FSR_FLAG_KEEP_INTERMEDIATES) != 0;
    const bool timing = (p.flags & FSR_FLAG_STAGE_TIMING) != 0;
    const uint64_t nn = std::max<uint32_t>(fp.n, 1);
    const uint64_t C = fp.C, nwords = fp.nwords;
    CK(h->keys0.ensure(4ull * nn));
    CK(h->vals0.ensure(4ull * nn));
    CK(h->keys1.ensure(4ull * nn));
    CK(h->vals1.ensure(4ull * nn));
    CK(h->radix_tmp.ensure(4ull * radix_scratch_words((uint32_t)nn)));
    CK(h->sorted.ensure(16ull * nn));
    CK(h->ranges.ensure(8ull * C));
    CK(h->occ.ensure(C));
    CK(h->surf.ensure(C));
    CK(h->bits.ensure(4ull * nwords + 4));
    CK(h->prefix.ensure(4ull * nwords + 4));
    const uint64_t G = (uint64_t)(fp.sp.res[0] + 1) * (fp.sp.res[1] + 1) * (fp.sp.res[2] + 1);
    CK(h->gflag.ensure(4ull * G));
    CK(h->glist.ensure(4ull * G));
    CK(h->ctr.ensure(sizeof(Counters)));
    if (yu13) {
        CK(h->invol.ensure(C));
        CK(h->cell_rmax.ensure(4ull * C));
        CK(h->mean.ensure(16ull * nn));
        CK(h->mean32.ensure(16ull * nn));
        CK(h->smoothed.ensure(16ull * nn));
        CK(h->grec.ensure(64ull * nn));
        CK(h->qrec.ensure(48ull * nn));
        CK(h->covrec.ensure(32ull * nn));
    }
    if (p.method == FSR_METHOD_AKINCI12) CK(h->psurf.ensure(nn));
    if (p.flags & FSR_FLAG_COMPUTE_DENSITY) CK(h->rho.ensure(4ull * nn));
    if (keep) CK(h->pflags.ensure(4ull * nn));
    if (!h->pinned_ctr) CK(cudaMallocHost(&h->pinned_ctr, sizeof(Counters)));
    if (timing && !h->ev_start) {
        CK(cudaEventCreate(&h->ev_start));
        for (auto& e : h->ev) CK(cudaEventCreate(&e));
    }
    const bool weld = (p.flags & FSR_FLAG_WELD) != 0;
    uint64_t scan_words = std::max<uint64_t>(scan_scratch_words(nwords), mc_offsets_scratch_words(h->cap_band));
    if (weld) {
        scan_words = std::max<uint64_t>(scan_words, scan_scratch_words(h->cap_mesh));
        const uint64_t cm = h->cap_mesh, ts = weld_table_size(h->cap_mesh);
        CK(h->wkey.ensure(8 * cm));
        CK(h->wslot.ensure(4 * cm));
        CK(h->wrank.ensure(4 * cm));
        CK(h->widx.ensure(4 * cm));
        CK(h->wpos.ensure(12 * cm));
        CK(h->wnrm.ensure(12 * cm));
        CK(h->wtable_keys.ensure(8 * ts));
        CK(h->wtable_first.ensure(4 * ts));
    }
    CK(h->scan_tmp.ensure(4ull * scan_words));
    CK(h->sv.ensure(4ull * h->cap_band));
    CK(h->phi.ensure(4ull * h->cap_band));
    CK(h->mc.ensure(4ull * h->cap_band));
    CK(h->vofs.ensure(4ull * h->cap_band));
    CK(h->valid.ensure(4ull * h->cap_valid));
    CK(h->mesh_pos.ensure(12ull * h->cap_mesh));
    CK(h->mesh_nrm.ensure(12ull * h->cap_mesh));
    if (!yu13 && p.method != FSR_METHOD_TC01) CK(h->mv.ensure(16ull * h->cap_band));
    return FSR_OK;
}

fsr_status frame_enqueue(fsr_handle* h, const FramePlan& fp, const float* d_xyz, const float* d_den,
                         cudaStream_t st, bool timing)
{
    const fsr_params& p = h->params;
    const fsr_frame_header& hdr = fp.hdr;
    const Grid sp = fp.sp, sc = fp.sc;
    const uint64_t C = fp.C;
    const uint32_t n = fp.n, nwords = fp.nwords;
    const bool yu13 = p.method == FSR_METHOD_YU13;
    const bool akinci = p.method == FSR_METHOD_AKINCI12;
    const bool keep = (p.flags & FSR_FLAG_KEEP_INTERMEDIATES) != 0;
    const KernelCtx kc{st, h->num_sms, h->grid_div, h->block};
    Counters* ctr = (Counters*)h->ctr.ptr;
    const float h_r = hdr.kernel_radius;
    const float h2 = h_r * h_r;

    auto mark = [&](int stage) {
        if (timing) cudaEventRecord(h->ev[stage], st);
    };
    if (timing) cudaEventRecord(h->ev_start, st);

    h->launches_mark = g_launches;
    CK(cudaMemsetAsync(ctr, 0, sizeof(Counters), st));
    CK(cudaMemsetAsync(h->ranges.ptr, 0xFF, 8ull * C, st));
    CK(cudaMemsetAsync(h->occ.ptr, 0, C, st));
    CK(cudaMemsetAsync(h->bits.ptr, 0, 4ull * nwords + 4, st));
    if (yu13) CK(cudaMemsetAsync(h->cell_rmax.ptr, 0, 4ull * C, st));

    // ---- spatial hashing (ReconstructorGPU.cpp:292-313)
    uint32_t* k0 = (uint32_t*)h->keys0.ptr;
    uint32_t* v0 = (uint32_t*)h->vals0.ptr;
    uint32_t* k1 = (uint32_t*)h->keys1.ptr;
    uint32_t* v1 = (uint32_t*)h->vals1.ptr;
    launch_hash(kc, d_xyz, n, sp, k0, v0, ctr);
    cudaError_t se = cudaSuccess;
    const int which = radix_sort_pairs(k0, v0, k1, v1, n, bits_for(C), (uint32_t*)h->radix_tmp.ptr, st, &se);
    if (se != cudaSuccess) return cuda_fail(h, se, "radix sort");
    const uint32_t* skeys = which ? k1 : k0;
    const uint32_t* perm = which ? v1 : v0;
    h->perm_ptr = perm;
    h->skeys_ptr = skeys;
    mark(0);
    float4* sorted = (float4*)h->sorted.ptr;
    uint2* ranges = (uint2*)h->ranges.ptr;
    uint8_t* occ = (uint8_t*)h->occ.ptr;
    const bool own_density = (p.flags & FSR_FLAG_COMPUTE_DENSITY) != 0;
    launch_ranges_gather(kc, skeys, perm, n, d_xyz, own_density ? nullptr : d_den, sorted, ranges, occ);
    if (own_density)
        launch_density(kc, sorted, n, ranges, sp, hdr.kernel_radius, hdr.particle_mass, (float*)h->rho.ptr);
    mark(1);

    // ---- surface cells / particles
    uint8_t* surf = (uint8_t*)h->surf.ptr;
    uint8_t* psurf = akinci ? (uint8_t*)h->psurf.ptr : nullptr;
    if (akinci) {
        launch_colorfield(kc, sorted, n, ranges, skeys, sp, h_r, h2, hdr.particle_mass, psurf);
    } else {
        launch_surface_cells(kc, sp, occ, surf);
        if (yu13) launch_involved_cells(kc, sp, occ, surf, (uint8_t*)h->invol.ptr);
    }
    if (keep) launch_particle_flags(kc, skeys, surf, psurf, n, (uint32_t*)h->pflags.ptr);
    mark(2);

    // ---- narrow band
    uint32_t* bits = (uint32_t*)h->bits.ptr;
    uint32_t* prefix = (uint32_t*)h->prefix.ptr;
    launch_band_stamp(kc, sorted, skeys, surf, psurf, n, sc, band_threshold(h_r), bits, ctr);
    mark(3);
    CK(scan_u32(bits, prefix, nwords, nullptr, nwords, &ctr->n_band, ScanInput::kPopcount,
                (uint32_t*)h->scan_tmp.ptr, st));
    uint32_t* sv = (uint32_t*)h->sv.ptr;
    const uint64_t G = (uint64_t)(sp.res[0] + 1) * (sp.res[1] + 1) * (sp.res[2] + 1);
    CK(cudaMemsetAsync(h->gflag.ptr, 0, 4ull * G, st));
    launch_band_list(kc, bits, prefix, nwords, sv, h->cap_band,
                     GroupMark{sp, sc, (uint32_t*)h->gflag.ptr, (uint32_t*)h->glist.ptr}, ctr);
    mark(4);

    // ---- field
    float* phi = (float*)h->phi.ptr;
    if (yu13) {
        const float R = h_r * p.aniso_radius_over_h;
        launch_smooth(kc, sorted, n, ranges, sp, R, p.smoothing_lambda, hdr.particle_mass, (float4*)h->mean.ptr,
                      (float4*)h->mean32.ptr, (float4*)h->smoothed.ptr);
        mark(5);
        CovArgs ca{};
        ca.sp = sp;
        ca.sorted = sorted;
        ca.mean = (const float4*)h->mean.ptr;
        ca.mean32 = (const float4*)h->mean32.ptr;
        ca.smoothed = (const float4*)h->smoothed.ptr;
        ca.ranges = ranges;
        ca.skeys = skeys;
        ca.invol = (const uint8_t*)h->invol.ptr;
        ca.grec = (float4*)h->grec.ptr;
        ca.qrec = (float4*)h->qrec.ptr;
        ca.crec = (float4*)h->covrec.ptr;
        ca.cell_rmax = (float*)h->cell_rmax.ptr;
        ca.n = n;
        ca.R = R;
        ca.h = h_r;
        ca.h2 = h2;
        ca.h_inv = (float)(1.0 / (double)h_r);
        ca.mass = hdr.particle_mass;
        ca.sigma = 315.0f / (64.0f * 3.1415926535898f);
        ca.min_neighbors = p.min_neighbors;
        launch_cov(kc, ca, ctr);
        mark(6);
        AnisoFieldArgs fa{};
        fa.sp = sp;
        fa.sc = sc;
        fa.smoothed = (const float4*)h->smoothed.ptr;
        fa.grec = (const float4*)h->grec.ptr;
        fa.qrec = (const float4*)h->qrec.ptr;
        fa.ranges = ranges;
        fa.invol = (const uint8_t*)h->invol.ptr;
        fa.occ = occ;
        fa.cell_rmax = (const float*)h->cell_rmax.ptr;
        fa.sv = sv;
        fa.phi = phi;
        fa.sigma = ca.sigma;
        fa.glist = (const uint32_t*)h->glist.ptr;
        fa.cap = h->cap_band;
        launch_field_aniso_grouped(kc, fa, BandView{bits, prefix, phi}, p.grid_ratio, ctr);
    } else {
        mark(5);
        mark(6);
        IsoFieldArgs fa{};
        fa.sp = sp;
        fa.sc = sc;
        fa.sorted = sorted;
        fa.skeys = skeys;
        fa.ranges = ranges;
        fa.sv = sv;
        fa.phi = phi;
        fa.h = h_r;
        fa.h2 = h2;
        fa.inv_h2 = 1.0f / h2;
        fa.rp = hdr.particle_radius;
        fa.mv = p.method == FSR_METHOD_TC01 ? nullptr : (float4*)h->mv.ptr;
        fa.glist = (const uint32_t*)h->glist.ptr;
        fa.cap = h->cap_band;
        launch_field_iso_grouped(kc, p.method == FSR_METHOD_TC01, fa, BandView{bits, prefix, phi}, p.grid_ratio, ctr);
    }
    mark(7);

    // ---- marching cubes
    McArgs ma{};
    ma.sc = sc;
    ma.band = BandView{bits, prefix, phi};
    ma.sv = sv;
    ma.mc = (uint32_t*)h->mc.ptr;
    ma.vofs = (uint32_t*)h->vofs.ptr;
    ma.valid = (uint32_t*)h->valid.ptr;
    ma.out_pos = (float*)h->mesh_pos.ptr;
    ma.out_nrm = (float*)h->mesh_nrm.ptr;
    ma.iso = p.iso_value;
    ma.fill = yu13 ? __builtin_bit_cast(float, 0x64646464u) : 0.0f;  // memset values (Yu13.cpp:264, ZB05.cpp:324)
    ma.host_mc = akinci ? 1 : 0;
    ma.cap_band = h->cap_band;
    ma.cap_valid = h->cap_valid;
    ma.cap_mesh = h->cap_mesh;
    const bool weld = (p.flags & FSR_FLAG_WELD) != 0;
    ma.out_key = weld ? (uint64_t*)h->wkey.ptr : nullptr;
    launch_mc_classify(kc, ma, ctr);
    mark(8);
    launch_mc_offsets(kc, ma, ctr, (uint32_t*)h->scan_tmp.ptr);
    mark(9);
    launch_mc_generate(kc, ma, ctr);
    if (weld) {
        WeldArgs wa{};
        wa.keys = (const uint64_t*)h->wkey.ptr;
        wa.pos = (const float*)h->mesh_pos.ptr;
        wa.nrm = (const float*)h->mesh_nrm.ptr;
        wa.cap = h->cap_mesh;
        wa.table_keys = (uint64_t*)h->wtable_keys.ptr;
        wa.table_first = (uint32_t*)h->wtable_first.ptr;
        wa.table_size = weld_table_size(h->cap_mesh);
        wa.slot = (uint32_t*)h->wslot.ptr;
        wa.rank = (uint32_t*)h->wrank.ptr;
        wa.index = (uint32_t*)h->widx.ptr;
        wa.out_pos = (float*)h->wpos.ptr;
        wa.out_nrm = (float*)h->wnrm.ptr;
        CK(launch_weld(kc, wa, ctr, (uint32_t*)h->scan_tmp.ptr));
    }
    mark(10);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->pinned_ctr, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    mark(11);
    h->launches_frame = (uint32_t)(g_launches - h->launches_mark);
    return FSR_OK;
}

fsr_status frame_finish(fsr_handle* h, const FramePlan& fp, bool timing, bool* retry)
{
    *retry = false;
    const Counters& hc = *h->pinned_ctr;
    if (hc.out_of_grid)
        return fail(h, FSR_ERR_OUT_OF_GRID, "%u particle(s) outside the expanded bounding box", hc.out_of_grid);
    if (hc.overflow) {
        if (hc.overflow & 1u)
            h->cap_band = (uint32_t)std::min<uint64_t>(fp.V, (uint64_t)hc.need_band * 5 / 4 + 1024);
        if (hc.overflow & 2u) h->cap_valid = std::min<uint32_t>(h->cap_band, hc.need_valid + hc.need_valid / 4 + 1024);
        if (hc.overflow & 4u)
            h->cap_mesh = (uint32_t)std::min<uint64_t>(0xFFFFFFF0ull, (uint64_t)hc.need_mesh * 5 / 4 + 4096);
        if (hc.overflow & 1u) {
            // a band overflow also invalidated the later stages' sizes
            h->cap_valid = std::max<uint32_t>(h->cap_valid, std::min<uint32_t>(h->cap_band, h->cap_band / 4));
        }
        h->stats.n_retries++;
        *retry = true;
        return FSR_OK;
    }
    fsr_stats& s = h->stats;
    s.n_particles = fp.n;
    s.n_cells = fp.C;
    s.n_grid_vertices = fp.V;
    s.n_surface_particles = hc.n_surface;
    s.n_involved_particles = hc.n_involved;
    s.n_band_vertices = hc.n_band;
    s.n_valid_cubes = hc.n_valid;
    s.n_mesh_vertices = hc.n_mesh_verts;
    s.n_weld_vertices = (h->params.flags & FSR_FLAG_WELD) ? hc.n_weld : 0;
    s.n_fp64_fallbacks = hc.n_fp64;
    s.n_kernel_launches = h->launches_frame;
    s.n_backward_launches = 0;
    s.device_bytes = 0;
    for (DevBuf* b : h->all_buffers()) s.device_bytes += b->bytes;
    for (int a = 0; a < 3; ++a) {
        s.spatial_res[a] = fp.sp.res[a];
        s.scalar_res[a] = fp.sc.res[a];
    }
    if (timing) {
        float prev = 0.f;
        for (int i = 0; i < FSR_NUM_STAGES; ++i) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, h->ev_start, h->ev[i]);
            s.stage_ms[i] = ms - prev;
            prev = ms;
        }
        s.total_ms = prev;
    }
    h->frame_ready = true;
    h->grid_sp = fp.sp;
    h->grid_sc = fp.sc;
    h->n_last = fp.n;
    h->C_last = fp.C;
    h->V_last = fp.V;
    h->hdr_last = fp.hdr;
    return FSR_OK;
}

fsr_status run_frame(fsr_handle* h, const fsr_frame_header& hdr, const float* d_xyz, const float* d_den,
                     uint64_t n64, cudaStream_t st)
{
    FramePlan fp;
    fsr_status s = frame_plan(h, hdr, n64, fp);
    if (s != FSR_OK) return s;
    const bool timing = (h->params.flags & FSR_FLAG_STAGE_TIMING) != 0;
    for (int attempt = 0; attempt < 4; ++attempt) {
        if ((s = frame_buffers(h, fp)) != FSR_OK) return s;
        if ((s = frame_enqueue(h, fp, d_xyz, d_den, st, timing)) != FSR_OK) return s;
        CK(cudaStreamSynchronize(st));
        bool retry = false;
        if ((s = frame_finish(h, fp, timing, &retry)) != FSR_OK || !retry) return s;
    }
    return fail(h, FSR_ERR_OUT_OF_MEMORY, "capacity growth did not converge");
}

}  // namespace fsr

// ------------------------------------------------------------ C ABI

extern "C" {

uint32_t fsr_abi_version(void) { return FSR_ABI_VERSION; }

const char* fsr_build_info(void)
{
    return "fsr_gb300 abi=1 arch=sm_103a";
}

fsr_status fsr_default_params(uint32_t method, fsr_params* out)
{
    if (!out || method > FSR_METHOD_AKINCI12) return FSR_ERR_INVALID_ARGUMENT;
    fsr_params p{};
    p.method = method;
    p.smoothing_lambda = 0.5f;
    p.aniso_radius_over_h = 2.0f;
    p.min_neighbors = 25;
    p.flags = 0;
    switch (method) {
    case FSR_METHOD_ZB05:  // ReconstructorGPUOursZB05.cpp:85-97
    case FSR_METHOD_AKINCI12:  // ReconstructorGPUAkinci12.cpp:93-106
        p.iso_value = -0.0001f;
        p.grid_ratio = 2;
        p.cell_size_scale = 1.0f;
        break;
    case FSR_METHOD_TC01:  // no reference caller: ZB05's grid, iso on the TC01 range [0, 1/4]
        p.iso_value = 0.25f;
        p.grid_ratio = 2;
        p.cell_size_scale = 1.0f;
        break;
    case FSR_METHOD_YU13:  // ReconstructorGPUOursYu13.cpp:78-99, anisotropic radius 2h at :21
        p.iso_value = 0.0f;
        p.grid_ratio = 3;
        p.cell_size_scale = 1.3f;
        break;
    }
    *out = p;
    return FSR_OK;
}

fsr_status fsr_create(const fsr_params* params, int device, fsr_handle** out)
{
    if (!params || !out) return FSR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!valid_params(*params)) return FSR_ERR_INVALID_ARGUMENT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return FSR_ERR_CUDA;
    }
    fsr_handle* h = new (std::nothrow) fsr_handle();
    if (!h) return FSR_ERR_OUT_OF_MEMORY;
    h->params = *params;
    h->device = device;
    DeviceGuard g(device);
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (h->num_sms <= 0) h->num_sms = 1;
    upload_mc_tables(0);
    cudaError_t e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) {
        delete h;
        return FSR_ERR_CUDA;
    }
    *out = h;
    return FSR_OK;
}

void fsr_destroy(fsr_handle* h) { delete h; }

fsr_status fsr_set_params(fsr_handle* h, const fsr_params* params)
{
    if (!h || !params) return FSR_ERR_INVALID_ARGUMENT;
    if (!valid_params(*params)) return fail(h, FSR_ERR_INVALID_ARGUMENT, "invalid parameters");
    h->params = *params;
    h->frame_ready = false;
    return FSR_OK;
}

const char* fsr_last_error(const fsr_handle* h) { return h ? h->last_error.c_str() : "null handle"; }

fsr_status fsr_reconstruct(fsr_handle* h, const fsr_frame_header* hdr, const float* d_xyz, const float* d_density,
                           uint64_t n, void* stream)
{
    if (!h || !hdr) return FSR_ERR_INVALID_ARGUMENT;
    const bool own_density = (h->params.flags & FSR_FLAG_COMPUTE_DENSITY) != 0;
    if (n > 0 && (!d_xyz || (!d_density && !own_density)))
        return fail(h, FSR_ERR_INVALID_ARGUMENT, "null particle arrays");
    DeviceGuard g(h->device);
    h->frame_ready = false;
    return run_frame(h, *hdr, d_xyz, d_density, n, (cudaStream_t)stream);
}

fsr_status fsr_reconstruct_host(fsr_handle* h, const fsr_frame_header* hdr, const float* xyz, const float* density,
                                uint64_t n, float* out_pos, float* out_nrm, uint64_t capacity, uint64_t* n_vertices,
                                void* stream)
{
    if (!h || !hdr || !n_vertices) return FSR_ERR_INVALID_ARGUMENT;
    const bool own_density = (h->params.flags & FSR_FLAG_COMPUTE_DENSITY) != 0;
    if (n > 0 && (!xyz || (!density && !own_density)))
        return fail(h, FSR_ERR_INVALID_ARGUMENT, "null particle arrays");
    DeviceGuard g(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    const uint64_t nn = std::max<uint64_t>(n, 1);
    CK(h->in_xyz.ensure(12ull * nn));
    CK(h->in_den.ensure(4ull * nn));
    if (n) {
        CK(cudaMemcpyAsync(h->in_xyz.ptr, xyz, 12ull * n, cudaMemcpyHostToDevice, st));
        if (!own_density) CK(cudaMemcpyAsync(h->in_den.ptr, density, 4ull * n, cudaMemcpyHostToDevice, st));
    }
    h->frame_ready = false;
    fsr_status s = run_frame(h, *hdr, (const float*)h->in_xyz.ptr, (const float*)h->in_den.ptr, n, st);
    if (s != FSR_OK) return s;
    const uint64_t nv = h->stats.n_mesh_vertices;
    *n_vertices = nv;
    if (nv > capacity) return fail(h, FSR_ERR_CAPACITY, "mesh has %llu vertices, buffer holds %llu",
                                   (unsigned long long)nv, (unsigned long long)capacity);
    if (nv) {
        if (!out_pos || !out_nrm) return fail(h, FSR_ERR_INVALID_ARGUMENT, "null mesh output");
        CK(cudaMemcpyAsync(out_pos, h->mesh_pos.ptr, 12ull * nv, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(out_nrm, h->mesh_nrm.ptr, 12ull * nv, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return FSR_OK;
}

fsr_status fsr_mesh_device(fsr_handle* h, const float** d_pos, const float** d_nrm, uint64_t* n_vertices)
{
    if (!h || !d_pos || !d_nrm || !n_vertices) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return fail(h, FSR_ERR_NOT_READY, "no frame reconstructed");
    *d_pos = (const float*)h->mesh_pos.ptr;
    *d_nrm = (const float*)h->mesh_nrm.ptr;
    *n_vertices = h->stats.n_mesh_vertices;
    return FSR_OK;
}

fsr_status fsr_copy_mesh(fsr_handle* h, float* out_pos, float* out_nrm, uint64_t capacity, uint64_t* n_vertices)
{
    if (!h || !n_vertices) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return fail(h, FSR_ERR_NOT_READY, "no frame reconstructed");
    DeviceGuard g(h->device);
    const uint64_t nv = h->stats.n_mesh_vertices;
    *n_vertices = nv;
    if (nv > capacity) return fail(h, FSR_ERR_CAPACITY, "mesh buffer too small");
    if (nv) {
        if (!out_pos || !out_nrm) return FSR_ERR_INVALID_ARGUMENT;
        CK(cudaMemcpy(out_pos, h->mesh_pos.ptr, 12ull * nv, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(out_nrm, h->mesh_nrm.ptr, 12ull * nv, cudaMemcpyDeviceToHost));
    }
    return FSR_OK;
}

fsr_status fsr_copy_indexed_mesh(fsr_handle* h, float* pos, float* nrm, uint64_t vertex_capacity, uint32_t* indices,
                                 uint64_t index_capacity, uint64_t* n_vertices, uint64_t* n_indices)
{
    if (!h || !n_vertices || !n_indices) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return fail(h, FSR_ERR_NOT_READY, "no frame reconstructed");
    if (!(h->params.flags & FSR_FLAG_WELD)) return fail(h, FSR_ERR_INVALID_ARGUMENT, "FSR_FLAG_WELD is not set");
    DeviceGuard g(h->device);
    const uint64_t nv = h->stats.n_weld_vertices, ni = h->stats.n_mesh_vertices;
    *n_vertices = nv;
    *n_indices = ni;
    if (nv > vertex_capacity || ni > index_capacity) return fail(h, FSR_ERR_CAPACITY, "indexed mesh buffers too small");
    if (nv) {
        if (!pos || !nrm || !indices) return FSR_ERR_INVALID_ARGUMENT;
        CK(cudaMemcpy(pos, h->wpos.ptr, 12ull * nv, cudaMemcpyDefault));
        CK(cudaMemcpy(nrm, h->wnrm.ptr, 12ull * nv, cudaMemcpyDefault));
        CK(cudaMemcpy(indices, h->widx.ptr, 4ull * ni, cudaMemcpyDefault));
    }
    return FSR_OK;
}

fsr_status fsr_get_stats(const fsr_handle* h, fsr_stats* out)
{
    if (!h || !out) return FSR_ERR_INVALID_ARGUMENT;
    *out = h->stats;
    return FSR_OK;
}

fsr_status fsr_get_frame_header(const fsr_handle* h, fsr_frame_header* out)
{
    if (!h || !out) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return FSR_ERR_NOT_READY;
    *out = h->hdr_last;
    return FSR_OK;
}

fsr_status fsr_debug_fetch(fsr_handle* h, uint32_t which, void* dst, uint64_t dst_bytes, uint64_t* bytes_needed)
{
    if (!h) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return fail(h, FSR_ERR_NOT_READY, "no frame reconstructed");
    DeviceGuard g(h->device);
    const uint64_t n = h->n_last, C = h->C_last;
    const fsr_stats& s = h->stats;
    const bool yu13 = h->params.method == FSR_METHOD_YU13;
    const bool keep = (h->params.flags & FSR_FLAG_KEEP_INTERMEDIATES) != 0;
    uint64_t need = 0;
    switch (which) {
    case FSR_DBG_SORT_PERM: need = 4 * n; break;
    case FSR_DBG_SORTED_XYZ: need = 12 * n; break;
    case FSR_DBG_CELL_RANGES: need = 8 * C; break;
    case FSR_DBG_SURFACE_FLAGS: need = keep ? 4 * n : 0; break;
    case FSR_DBG_INVOLVED_COUNTS: need = yu13 ? 4 * C : 0; break;
    case FSR_DBG_BAND_VERTICES:
    case FSR_DBG_FIELD:
    case FSR_DBG_MC_INFO: need = 4 * s.n_band_vertices; break;
    case FSR_DBG_VALID_CUBES: need = 4 * s.n_valid_cubes; break;
    case FSR_DBG_MEAN:
    case FSR_DBG_SMOOTHED: need = yu13 ? 12 * n : 0; break;
    case FSR_DBG_G: need = yu13 ? 36 * n : 0; break;
    case FSR_DBG_WELD_KEYS: need = (h->params.flags & FSR_FLAG_WELD) ? 8 * s.n_mesh_vertices : 0; break;
    case FSR_DBG_DENSITY: need = 4 * n; break;
    default: return fail(h, FSR_ERR_INVALID_ARGUMENT, "unknown debug array %u", which);
    }
    if (bytes_needed) *bytes_needed = need;
    if (!dst) return FSR_OK;
    if (dst_bytes < need) return fail(h, FSR_ERR_CAPACITY, "debug buffer too small");
    if (need == 0) return FSR_OK;
    auto copy4 = [&](const DevBuf& b, size_t stride_floats, size_t take, size_t count, float* out) -> cudaError_t {
        std::vector<float> tmp(stride_floats * count);
        cudaError_t e = cudaMemcpy(tmp.data(), b.ptr, 4 * tmp.size(), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return e;
        for (size_t i = 0; i < count; ++i)
            for (size_t k = 0; k < take; ++k) out[take * i + k] = tmp[stride_floats * i + k];
        return cudaSuccess;
    };
    switch (which) {
    case FSR_DBG_SORT_PERM: CK(cudaMemcpy(dst, h->perm_ptr, need, cudaMemcpyDeviceToHost)); break;
    case FSR_DBG_SORTED_XYZ: CK(copy4(h->sorted, 4, 3, n, (float*)dst)); break;
    case FSR_DBG_CELL_RANGES: CK(cudaMemcpy(dst, h->ranges.ptr, need, cudaMemcpyDeviceToHost)); break;
    case FSR_DBG_SURFACE_FLAGS: CK(cudaMemcpy(dst, h->pflags.ptr, need, cudaMemcpyDeviceToHost)); break;
    case FSR_DBG_INVOLVED_COUNTS: {
        std::vector<uint8_t> inv(C);
        std::vector<uint32_t> rg(2 * C);
        CK(cudaMemcpy(inv.data(), h->invol.ptr, C, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(rg.data(), h->ranges.ptr, 8 * C, cudaMemcpyDeviceToHost));
        uint32_t* o = (uint32_t*)dst;
        for (uint64_t c = 0; c < C; ++c) o[c] = inv[c] ? rg[2 * c + 1] - rg[2 * c] : 0u;
        break;
    }
    case FSR_DBG_BAND_VERTICES: CK(cudaMemcpy(dst, h->sv.ptr, need, cudaMemcpyDeviceToHost)); break;
    case FSR_DBG_FIELD: CK(cudaMemcpy(dst, h->phi.ptr, need, cudaMemcpyDeviceToHost)); break;
    case FSR_DBG_MC_INFO: {
        CK(cudaMemcpy(dst, h->mc.ptr, need, cudaMemcpyDeviceToHost));
        uint32_t* o = (uint32_t*)dst;
        for (uint64_t i = 0; i < s.n_band_vertices; ++i) {
            const uint32_t nv = o[i] & 0xFFu;
            o[i] = (o[i] >> 8) | (nv << 8) | ((nv ? 1u : 0u) << 16);
        }
        break;
    }
    case FSR_DBG_VALID_CUBES: CK(cudaMemcpy(dst, h->valid.ptr, need, cudaMemcpyDeviceToHost)); break;
    case FSR_DBG_WELD_KEYS: CK(cudaMemcpy(dst, h->wkey.ptr, need, cudaMemcpyDeviceToHost)); break;
    case FSR_DBG_DENSITY: {
        std::vector<float> tmp(4 * n);
        CK(cudaMemcpy(tmp.data(), h->sorted.ptr, 16 * n, cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < n; ++i) ((float*)dst)[i] = tmp[4 * i + 3];
        break;
    }
    case FSR_DBG_MEAN: CK(copy4(h->mean32, 4, 3, n, (float*)dst)); break;
    case FSR_DBG_SMOOTHED: CK(copy4(h->smoothed, 4, 3, n, (float*)dst)); break;
    case FSR_DBG_G: {
        std::vector<float> tmp(16 * n);
        CK(cudaMemcpy(tmp.data(), h->grec.ptr, 64 * n, cudaMemcpyDeviceToHost));
        float* o = (float*)dst;
        for (uint64_t i = 0; i < n; ++i) {
            const float* r = &tmp[16 * i];
            const float g[9] = {r[4], r[5], r[6], r[8], r[9], r[10], r[12], r[13], r[14]};
            for (int k = 0; k < 9; ++k) o[9 * i + k] = g[k];
        }
        break;
    }
    }
    return FSR_OK;
}

}  // extern "C"
