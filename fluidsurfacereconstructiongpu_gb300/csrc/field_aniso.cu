// Anisotropic field, grouped by window (computationOfScalarFieldGrid,
// ReconstructionCUDA.cu:830-906).
//
// A band vertex's candidate particles are the particles of the +-2 cells
// around the spatial cell its FP32 position falls in; every vertex that
// falls in the same cell has the same window.  Along each axis that cell
// index is a non-decreasing function of the vertex index, so the vertices
// of one cell form an index box, found exactly without sorting.  One block
// handles one such group:
//   1. it lists the group's band vertices (bitset tests, order kept per
//      warp) and their rank in the band;
//   2. it lists the window's candidate cells, dropping involved cells that
//      lie beyond the reach (largest support radius + smoothing shift) of all
//      their particles from the group's vertex box;
//   3. it streams the candidates through shared memory in chunks of 256
//      records; each warp keeps the candidates whose support can reach the
//      bounding box of its own vertices, and each lane evaluates only those.
// Particles of non-involved cells use the unscaled kernel (cuh:312-322),
// written here as G = I with support 1, so one evaluation path serves both.
// Only terms that are exactly zero are skipped; the summation order is the
// candidate order, the same for every vertex, so results are deterministic.
#include "kernels.h"

#include <algorithm>

namespace fsr {
namespace {

constexpr int kBT = 256;            // threads per block
constexpr int kWarps = kBT / 32;
constexpr int kChunk = 256;         // candidate records per shared-memory chunk
constexpr int kMaxCells = 125;      // 5 x 5 x 5 window

struct GroupArgs {
    Grid sp, sc;
    BandView band;
    const float4* grec;
    const float4* smoothed;
    const uint2* ranges;
    const uint8_t* invol;
    const float* reach;
    float* phi;
    float sigma;
    uint32_t cap;
    uint32_t vlist_cap;             // capacity of the per-block vertex list
};

__global__ void k_field_aniso_grouped(GroupArgs a, uint32_t ratio, const Counters* ctr)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float4* rec = reinterpret_cast<float4*>(smem);                         // kChunk * 4 float4
    uint16_t* wlist = reinterpret_cast<uint16_t*>(rec + 4 * kChunk);       // kWarps * kChunk
    uint32_t* cstart = reinterpret_cast<uint32_t*>(wlist + kWarps * kChunk);
    uint32_t* cpre = cstart + 128;                                         // prefix over candidate cells
    uint32_t* cinv = cpre + 129;
    uint32_t* vrank = cinv + 128;                                          // vertex list: rank
    uint32_t* vid = vrank + a.vlist_cap;                                   // vertex list: grid vertex id
    __shared__ uint32_t s_nv, s_tot, s_wsum[4];

    const uint32_t nb = min(ctr->n_band, a.cap);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int kx = (int)a.sp.res[0] + 1, ky = (int)a.sp.res[1] + 1, kz = (int)a.sp.res[2] + 1;
    const uint32_t ngroups = (uint32_t)kx * ky * kz;

    for (uint32_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int cx = (int)(g % kx), cy = (int)((g / kx) % ky), cz = (int)(g / ((uint32_t)kx * ky));
        const int x0 = first_vertex<0>(cx, a.sc, a.sp, ratio), x1 = first_vertex<0>(cx + 1, a.sc, a.sp, ratio);
        const int y0 = first_vertex<1>(cy, a.sc, a.sp, ratio), y1 = first_vertex<1>(cy + 1, a.sc, a.sp, ratio);
        const int z0 = first_vertex<2>(cz, a.sc, a.sp, ratio), z1 = first_vertex<2>(cz + 1, a.sc, a.sp, ratio);
        const int nx = x1 - x0, ny = y1 - y0, nz = z1 - z0;
        if (nx <= 0 || ny <= 0 || nz <= 0) continue;  // uniform across the block
        const int nbox = nx * ny * nz;

        // 1. the group's band vertices, in box order within each warp
        if (tid == 0) s_nv = 0;
        __syncthreads();
        for (int base = 0; base < nbox; base += kBT) {
            const int i = base + tid;
            bool in = false;
            uint32_t v = 0;
            if (i < nbox) {
                const int lx = i % nx, ly = (i / nx) % ny, lz = i / (nx * ny);
                v = lin3(x0 + lx, y0 + ly, z0 + lz, a.sc);
                in = band_has(a.band, v);
            }
            const uint32_t m = __ballot_sync(0xffffffffu, in);
            uint32_t off = 0;
            if (lane == 0 && m) off = atomicAdd(&s_nv, __popc(m));
            off = __shfl_sync(0xffffffffu, off, 0);
            if (in) {
                const uint32_t slot = off + __popc(m & ((1u << lane) - 1u));
                if (slot < a.vlist_cap) {
                    vid[slot] = v;
                    vrank[slot] = band_rank(a.band, v);
                }
            }
        }
        __syncthreads();
        const uint32_t nv = min(s_nv, a.vlist_cap);
        if (nv == 0) continue;

        // 2. candidate cells of the window (clamped as in the reference)
        const int lx = clampi(cx - 2, 0, (int)a.sp.res[0] - 1), hx = clampi(cx + 2, 0, (int)a.sp.res[0] - 1);
        const int ly = clampi(cy - 2, 0, (int)a.sp.res[1] - 1), hy = clampi(cy + 2, 0, (int)a.sp.res[1] - 1);
        const int lz = clampi(cz - 2, 0, (int)a.sp.res[2] - 1), hz = clampi(cz + 2, 0, (int)a.sp.res[2] - 1);
        const float bx0 = vpos1(x0, a.sc.min[0], a.sc.cs), bx1 = vpos1(x1 - 1, a.sc.min[0], a.sc.cs);
        const float by0 = vpos1(y0, a.sc.min[1], a.sc.cs), by1 = vpos1(y1 - 1, a.sc.min[1], a.sc.cs);
        const float bz0 = vpos1(z0, a.sc.min[2], a.sc.cs), bz1 = vpos1(z1 - 1, a.sc.min[2], a.sc.cs);
        uint32_t cnt = 0;
        if (tid < kMaxCells) {
            const int dx = tid % 5, dy = (tid / 5) % 5, dz = tid / 25;
            const int xx = lx + dx, yy = ly + dy, zz = lz + dz;
            uint32_t st = 0, inv = 0;
            if (xx <= hx && yy <= hy && zz <= hz) {
                const uint32_t c = lin3(xx, yy, zz, a.sp);
                const uint2 r = __ldg(&a.ranges[c]);
                if (r.x != kEmpty) {
                    inv = __ldg(&a.invol[c]);
                    bool keep = true;
                    if (inv) {
                        const float cs = a.sp.cs;
                        const float cx0 = a.sp.min[0] + xx * cs, cy0 = a.sp.min[1] + yy * cs, cz0 = a.sp.min[2] + zz * cs;
                        const float gx = fmaxf(0.f, fmaxf(cx0 - bx1, bx0 - (cx0 + cs)));
                        const float gy = fmaxf(0.f, fmaxf(cy0 - by1, by0 - (cy0 + cs)));
                        const float gz = fmaxf(0.f, fmaxf(cz0 - bz1, bz0 - (cz0 + cs)));
                        const float cr = cull_radius(__ldg(&a.reach[c]), cs);
                        keep = fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < cr * cr;
                    }
                    if (keep) {
                        st = r.x;
                        cnt = r.y - r.x;
                    }
                }
            }
            cstart[tid] = st;
            cinv[tid] = inv;
        }
        // block-wide exclusive scan of the candidate counts (125 entries, warps 0-3)
        uint32_t x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (warp < 4 && lane == 31) s_wsum[warp] = x;
        __syncthreads();
        if (warp < 4) {
            uint32_t off = 0;
            for (int w = 0; w < warp; ++w) off += s_wsum[w];
            cpre[tid + 1] = x + off;
        }
        if (tid == 0) cpre[0] = 0;
        __syncthreads();
        if (tid == 0) s_tot = cpre[kMaxCells];
        __syncthreads();
        const uint32_t total = s_tot;

        // 3. vertex passes; candidates streamed per pass
        for (uint32_t vb = 0; vb < nv; vb += kBT) {
            const bool have = vb + tid < nv;
            uint32_t rank = 0;
            float vx = 0.f, vy = 0.f, vz = 0.f;
            if (have) {
                rank = vrank[vb + tid];
                uint32_t x, y, z;
                unlin3(vid[vb + tid], a.sc, x, y, z);
                vx = vpos1(x, a.sc.min[0], a.sc.cs);
                vy = vpos1(y, a.sc.min[1], a.sc.cs);
                vz = vpos1(z, a.sc.min[2], a.sc.cs);
            }
            // bounding box of this warp's vertices
            float mnx = have ? vx : 3.0e38f, mny = have ? vy : 3.0e38f, mnz = have ? vz : 3.0e38f;
            float mxx = have ? vx : -3.0e38f, mxy = have ? vy : -3.0e38f, mxz = have ? vz : -3.0e38f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
                mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
                mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, o));
                mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
                mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
                mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
            }
            const bool warp_active = __any_sync(0xffffffffu, have);
            float sum = 0.f;
            for (uint32_t cb = 0; cb < total; cb += kChunk) {
                // load one candidate record per thread
                const uint32_t j = cb + tid;
                if (j < total) {
                    int lo = 0, hi = kMaxCells;  // find k with cpre[k] <= j < cpre[k+1]
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (cpre[mid] <= j) lo = mid;
                        else hi = mid;
                    }
                    const uint32_t i = cstart[lo] + (j - cpre[lo]);
                    float4* r = rec + 4 * tid;
                    if (cinv[lo]) {
                        const float4* gsrc = a.grec + 4ull * i;
                        r[0] = __ldg(gsrc);
                        r[1] = __ldg(gsrc + 1);
                        r[2] = __ldg(gsrc + 2);
                        r[3] = __ldg(gsrc + 3);
                    } else {
                        const float4 s = __ldg(&a.smoothed[i]);
                        r[0] = make_float4(s.x, s.y, s.z, 1.0f);
                        r[1] = make_float4(1.f, 0.f, 0.f, a.sigma * s.w);
                        r[2] = make_float4(0.f, 1.f, 0.f, 0.f);
                        r[3] = make_float4(0.f, 0.f, 1.f, 0.f);
                    }
                }
                __syncthreads();
                const uint32_t cn = min((uint32_t)kChunk, total - cb);
                if (warp_active) {
                    // candidates whose support reaches this warp's vertex box
                    uint32_t wc = 0;
                    uint16_t* mylist = wlist + warp * kChunk;
                    for (uint32_t q = 0; q < cn; q += 32) {
                        const uint32_t idx = q + lane;
                        bool keep = false;
                        if (idx < cn) {
                            const float4 r0 = rec[4 * idx];
                            const float gx = fmaxf(0.f, fmaxf(mnx - r0.x, r0.x - mxx));
                            const float gy = fmaxf(0.f, fmaxf(mny - r0.y, r0.y - mxy));
                            const float gz = fmaxf(0.f, fmaxf(mnz - r0.z, r0.z - mxz));
                            keep = fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < r0.w;
                        }
                        const uint32_t m = __ballot_sync(0xffffffffu, keep);
                        if (keep) mylist[wc + __popc(m & ((1u << lane) - 1u))] = (uint16_t)idx;
                        wc += __popc(m);
                    }
                    __syncwarp();
                    if (have) {
                        for (uint32_t k = 0; k < wc; ++k) {
                            const float4* r = rec + 4 * mylist[k];
                            const float4 r0 = r[0];
                            const float rx = r0.x - vx, ry = r0.y - vy, rz = r0.z - vz;
                            const float d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                            if (d2 < r0.w) {
                                const float4 g0 = r[1], g1 = r[2], g2 = r[3];
                                const float tx = fmaf(g0.x, rx, fmaf(g0.y, ry, g0.z * rz));
                                const float ty = fmaf(g1.x, rx, fmaf(g1.y, ry, g1.z * rz));
                                const float tz = fmaf(g2.x, rx, fmaf(g2.y, ry, g2.z * rz));
                                const float q2 = fmaf(tx, tx, fmaf(ty, ty, tz * tz));
                                if (q2 < 1.0f) {
                                    const float u = 1.0f - q2;
                                    sum = fmaf(g0.w, u * u * u, sum);
                                }
                            }
                        }
                    }
                }
                __syncthreads();
            }
            if (have && rank < nb) a.phi[rank] = sum - 0.5f;
        }
    }
}

}  // namespace

bool launch_field_aniso_grouped(const KernelCtx& c, const AnisoFieldArgs& f, const BandView& band, uint32_t ratio,
                                Counters* ctr)
{
    // the group's index box is at most (ratio + 2)^3 vertices
    const uint32_t vcap = (ratio + 2) * (ratio + 2) * (ratio + 2);
    const size_t smem = sizeof(float4) * 4 * kChunk + sizeof(uint16_t) * kWarps * kChunk +
                        sizeof(uint32_t) * (128 + 129 + 128) + sizeof(uint32_t) * 2 * vcap;
    if (smem > 200 * 1024) return false;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_field_aniso_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        configured = true;
    }
    GroupArgs a;
    a.sp = f.sp;
    a.sc = f.sc;
    a.band = band;
    a.grec = f.grec;
    a.smoothed = f.smoothed;
    a.ranges = f.ranges;
    a.invol = f.invol;
    a.reach = f.cell_rmax;
    a.phi = f.phi;
    a.sigma = f.sigma;
    a.cap = f.cap;
    a.vlist_cap = vcap;
    const uint64_t groups = (uint64_t)(f.sp.res[0] + 1) * (f.sp.res[1] + 1) * (f.sp.res[2] + 1);
    const unsigned grid = (unsigned)std::min<uint64_t>(groups, (uint64_t)c.num_sms * 8);
    k_field_aniso_grouped<<<grid, kBT, smem, c.stream>>>(a, ratio, ctr);
    ++g_launches;
    return true;
}

}  // namespace fsr
