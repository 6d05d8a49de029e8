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
#ifndef FSR_FIELD_CHUNK
#define FSR_FIELD_CHUNK 128
#endif
constexpr int kChunk = FSR_FIELD_CHUNK;  // candidate records per shared-memory chunk (a multiple of 32)
static_assert(kChunk % 32 == 0 && kChunk <= 65536, "chunk indices are 16-bit, warp lists step by 32");
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

// Shared-memory tables of one group's candidate cells.
struct CandTables {
    uint32_t* cstart;  // first sorted particle of each window cell (kMaxCells)
    uint32_t* cpre;    // exclusive prefix of the kept cells' particle counts (kMaxCells + 1)
    uint32_t* cinv;    // the cell is involved (its particles carry a G record)
};

// Group g (a key of the (res + 1)^3 window-centre grid): its cell and its
// vertex index box [x0, x1) x [y0, y1) x [z0, z1).
__device__ __forceinline__ bool group_box(uint32_t g, const Grid& sp, const Grid& sc, uint32_t ratio, int c[3],
                                          int lo[3], int hi[3])
{
    const uint32_t kx = sp.res[0] + 1, ky = sp.res[1] + 1;
    c[0] = (int)(g % kx);
    c[1] = (int)((g / kx) % ky);
    c[2] = (int)(g / (kx * ky));
    lo[0] = first_vertex<0>(c[0], sc, sp, ratio);
    hi[0] = first_vertex<0>(c[0] + 1, sc, sp, ratio);
    lo[1] = first_vertex<1>(c[1], sc, sp, ratio);
    hi[1] = first_vertex<1>(c[1] + 1, sc, sp, ratio);
    lo[2] = first_vertex<2>(c[2], sc, sp, ratio);
    hi[2] = first_vertex<2>(c[2] + 1, sc, sp, ratio);
    return hi[0] > lo[0] && hi[1] > lo[1] && hi[2] > lo[2];
}

// Lists the candidate cells of the window around cell c (clamped as in the
// reference, cu:856-864), dropping involved cells whose reach cannot touch
// the box [b0, b1], and scans their particle counts.  Every thread of the
// block calls it; returns the number of candidates.
__device__ uint32_t group_candidates(const Grid& sp, const uint2* __restrict__ ranges,
                                     const uint8_t* __restrict__ invol, const float* __restrict__ reach,
                                     const int c[3], const float b0[3], const float b1[3], const CandTables& t,
                                     uint32_t* s_wsum, uint32_t* s_tot)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int lx = clampi(c[0] - 2, 0, (int)sp.res[0] - 1), hx = clampi(c[0] + 2, 0, (int)sp.res[0] - 1);
    const int ly = clampi(c[1] - 2, 0, (int)sp.res[1] - 1), hy = clampi(c[1] + 2, 0, (int)sp.res[1] - 1);
    const int lz = clampi(c[2] - 2, 0, (int)sp.res[2] - 1), hz = clampi(c[2] + 2, 0, (int)sp.res[2] - 1);
    uint32_t cnt = 0;
    if (tid < kMaxCells) {
        const int dx = tid % 5, dy = (tid / 5) % 5, dz = tid / 25;
        const int xx = lx + dx, yy = ly + dy, zz = lz + dz;
        uint32_t st = 0, inv = 0;
        if (xx <= hx && yy <= hy && zz <= hz) {
            const uint32_t cell = lin3(xx, yy, zz, sp);
            const uint2 r = __ldg(&ranges[cell]);
            if (r.x != kEmpty) {
                inv = __ldg(&invol[cell]);
                bool keep = true;
                if (inv) {
                    const float cs = sp.cs;
                    const float cx0 = sp.min[0] + xx * cs, cy0 = sp.min[1] + yy * cs, cz0 = sp.min[2] + zz * cs;
                    const float gx = fmaxf(0.f, fmaxf(cx0 - b1[0], b0[0] - (cx0 + cs)));
                    const float gy = fmaxf(0.f, fmaxf(cy0 - b1[1], b0[1] - (cy0 + cs)));
                    const float gz = fmaxf(0.f, fmaxf(cz0 - b1[2], b0[2] - (cz0 + cs)));
                    const float cr = cull_radius(__ldg(&reach[cell]), cs);
                    keep = fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < cr * cr;
                }
                if (keep) {
                    st = r.x;
                    cnt = r.y - r.x;
                }
            }
        }
        t.cstart[tid] = st;
        t.cinv[tid] = inv;
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
        t.cpre[tid + 1] = x + off;
    }
    if (tid == 0) t.cpre[0] = 0;
    __syncthreads();
    if (tid == 0) *s_tot = t.cpre[kMaxCells];
    __syncthreads();
    return *s_tot;
}

// Candidate j of the group: its sorted particle index and window cell.
__device__ __forceinline__ uint32_t candidate(uint32_t j, const CandTables& t, int* cell)
{
    int lo = 0, hi = kMaxCells;  // find k with cpre[k] <= j < cpre[k+1]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (t.cpre[mid] <= j) lo = mid;
        else hi = mid;
    }
    *cell = lo;
    return t.cstart[lo] + (j - t.cpre[lo]);
}

// The 4 float4 field record of particle i: (x~, r2max), G rows with
// coef = sigma det(G) m / rho in the first row's w; non-involved particles
// get G = I, support 1 and coef = sigma m / rho.
__device__ __forceinline__ void load_record(const float4* __restrict__ grec, const float4* __restrict__ smoothed,
                                            float sigma, uint32_t i, bool involved, float4 r[4])
{
    if (involved) {
        const float4* gsrc = grec + 4ull * i;
        r[0] = __ldg(gsrc);
        r[1] = __ldg(gsrc + 1);
        r[2] = __ldg(gsrc + 2);
        r[3] = __ldg(gsrc + 3);
    } else {
        const float4 s = __ldg(&smoothed[i]);
        r[0] = make_float4(s.x, s.y, s.z, 1.0f);
        r[1] = make_float4(1.f, 0.f, 0.f, sigma * s.w);
        r[2] = make_float4(0.f, 1.f, 0.f, 0.f);
        r[3] = make_float4(0.f, 0.f, 1.f, 0.f);
    }
}

__global__ void k_field_aniso_grouped(GroupArgs a, uint32_t ratio, const Counters* ctr)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t ntile_cap = (a.vlist_cap + 31) / 32;
    float4* rec = reinterpret_cast<float4*>(smem);                         // kChunk * 4 float4
    float4* tbox = rec + 4 * kChunk;                                       // per 32-vertex tile: lo, hi
    uint32_t* vid = reinterpret_cast<uint32_t*>(tbox + 2 * ntile_cap);     // vertex list: grid vertex id
    uint32_t* vrank = vid + a.vlist_cap;                                   // vertex list: band rank
    float* vsum = reinterpret_cast<float*>(vrank + a.vlist_cap);           // per vertex partial sum
    uint16_t* wlist = reinterpret_cast<uint16_t*>(vsum + a.vlist_cap);     // kWarps * kChunk
    uint32_t* cstart = reinterpret_cast<uint32_t*>(wlist + kWarps * kChunk);
    uint32_t* cpre = cstart + 128;                                         // prefix over candidate cells
    uint32_t* cinv = cpre + 129;
    __shared__ uint32_t s_nv, s_tot, s_wsum[4];
    const CandTables tabs{cstart, cpre, cinv};

    const uint32_t nb = min(ctr->n_band, a.cap);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t ngroups = (a.sp.res[0] + 1) * (a.sp.res[1] + 1) * (a.sp.res[2] + 1);

    for (uint32_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
        int c[3], lo[3], hi[3];
        if (!group_box(g, a.sp, a.sc, ratio, c, lo, hi)) continue;  // uniform across the block
        const int nx = hi[0] - lo[0], ny = hi[1] - lo[1], nz = hi[2] - lo[2];
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
                v = lin3(lo[0] + lx, lo[1] + ly, lo[2] + lz, a.sc);
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
                    vsum[slot] = 0.f;
                }
            }
        }
        __syncthreads();
        const uint32_t nv = min(s_nv, a.vlist_cap);
        if (nv == 0) continue;
        const uint32_t ntiles = (nv + 31) / 32;
        auto vertex_pos = [&](uint32_t q) {
            uint32_t x, y, z;
            unlin3(vid[q], a.sc, x, y, z);
            return make_float3(vpos1(x, a.sc.min[0], a.sc.cs), vpos1(y, a.sc.min[1], a.sc.cs),
                               vpos1(z, a.sc.min[2], a.sc.cs));
        };
        for (uint32_t t = tid; t < ntiles; t += kBT) {
            float4 l = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f), h = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
            for (uint32_t q = 32 * t; q < min(nv, 32 * t + 32); ++q) {
                const float3 v = vertex_pos(q);
                l.x = fminf(l.x, v.x); l.y = fminf(l.y, v.y); l.z = fminf(l.z, v.z);
                h.x = fmaxf(h.x, v.x); h.y = fmaxf(h.y, v.y); h.z = fmaxf(h.z, v.z);
            }
            tbox[2 * t] = l;
            tbox[2 * t + 1] = h;
        }

        // 2. candidate cells of the window
        const float b0[3] = {vpos1(lo[0], a.sc.min[0], a.sc.cs), vpos1(lo[1], a.sc.min[1], a.sc.cs),
                             vpos1(lo[2], a.sc.min[2], a.sc.cs)};
        const float b1[3] = {vpos1(hi[0] - 1, a.sc.min[0], a.sc.cs), vpos1(hi[1] - 1, a.sc.min[1], a.sc.cs),
                             vpos1(hi[2] - 1, a.sc.min[2], a.sc.cs)};
        const uint32_t total = group_candidates(a.sp, a.ranges, a.invol, a.reach, c, b0, b1, tabs, s_wsum, &s_tot);

        // 3. candidates streamed once through shared memory; per chunk the
        //    warps take the group's 32-vertex tiles round robin, each keeping
        //    the candidates whose support reaches its tile's box
        for (uint32_t cb = 0; cb < total; cb += kChunk) {
            for (uint32_t q = tid; q < (uint32_t)kChunk; q += kBT) {
                const uint32_t j = cb + q;
                if (j < total) {
                    int cell;
                    const uint32_t i = candidate(j, tabs, &cell);
                    float4 r[4];
                    load_record(a.grec, a.smoothed, a.sigma, i, cinv[cell] != 0, r);
                    float4* dst = rec + 4 * q;
                    dst[0] = r[0];
                    dst[1] = r[1];
                    dst[2] = r[2];
                    dst[3] = r[3];
                }
            }
            __syncthreads();
            const uint32_t cn = min((uint32_t)kChunk, total - cb);
            uint16_t* mylist = wlist + warp * kChunk;
            for (uint32_t t = warp; t < ntiles; t += kWarps) {
                const float4 tl = tbox[2 * t], th = tbox[2 * t + 1];
                uint32_t wc = 0;
                for (uint32_t q = 0; q < cn; q += 32) {
                    const uint32_t idx = q + lane;
                    bool keep = false;
                    if (idx < cn) {
                        const float4 r0 = rec[4 * idx];
                        const float gx = fmaxf(0.f, fmaxf(tl.x - r0.x, r0.x - th.x));
                        const float gy = fmaxf(0.f, fmaxf(tl.y - r0.y, r0.y - th.y));
                        const float gz = fmaxf(0.f, fmaxf(tl.z - r0.z, r0.z - th.z));
                        keep = fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < r0.w;
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, keep);
                    if (keep) mylist[wc + __popc(m & ((1u << lane) - 1u))] = (uint16_t)idx;
                    wc += __popc(m);
                }
                __syncwarp();
                const uint32_t v = 32 * t + lane;
                if (wc && v < nv) {
                    const float3 vp = vertex_pos(v);
                    float sum = vsum[v];
                    for (uint32_t k = 0; k < wc; ++k) {
                        const float4* r = rec + 4 * mylist[k];
                        const float4 r0 = r[0];
                        const float rx = r0.x - vp.x, ry = r0.y - vp.y, rz = r0.z - vp.z;
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
                    vsum[v] = sum;
                }
                __syncwarp();
            }
            __syncthreads();
        }
        for (uint32_t v = tid; v < nv; v += kBT) {
            const uint32_t rank = vrank[v];
            if (rank < nb) a.phi[rank] = vsum[v] - 0.5f;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- adjoint
// dL/dx~ and dL/dG of the anisotropic field, grouped like the forward pass
// but with the roles swapped: the group's band vertices that carry a
// non-zero dL/dphi are staged in shared memory (with one bounding box per
// 32 of them), and each thread takes one candidate particle, walks those
// vertices and keeps its partial gradient in registers; one float4 atomic
// per row then adds it to the particle (a particle is a candidate of up to
// 125 groups).  Per (vertex, particle) pair inside the support:
//   phi += c (1 - q2)^3, q2 = |G r|^2, r = x~ - v
//   dL/dx~ += g c (-6 (1 - q2)^2) G^T G r,  dL/dG += g c (-6 (1 - q2)^2) (G r) r^T
//   and sum g (1 - q2)^3 into the w of the dL/dx~ row (the det(G) term of
//   c = sigma det(G) m / rho is applied per particle afterwards).
struct BwdGroupArgs {
    Grid sp, sc;
    BandView band;
    const float4* grec;
    const float4* smoothed;
    const uint2* ranges;
    const uint8_t* invol;
    const float* reach;
    const float* gphi;
    const uint8_t* gkey;
    float4* gsmooth;
    float4* gG;
    float sigma;
    uint32_t cap;
    uint32_t vlist_cap;
};

__device__ __forceinline__ float box_dist2(float x, float y, float z, float4 lo, float4 hi)
{
    const float gx = fmaxf(0.f, fmaxf(lo.x - x, x - hi.x));
    const float gy = fmaxf(0.f, fmaxf(lo.y - y, y - hi.y));
    const float gz = fmaxf(0.f, fmaxf(lo.z - z, z - hi.z));
    return fmaf(gx, gx, fmaf(gy, gy, gz * gz));
}

__global__ void k_field_aniso_backward_grouped(BwdGroupArgs a, uint32_t ratio, const Counters* ctr)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t nch_cap = (a.vlist_cap + 31) / 32;
    float4* av = reinterpret_cast<float4*>(smem);            // active vertices: (v, dL/dphi)
    float4* cbox = av + a.vlist_cap;                          // per 32 of them: lo, hi
    uint32_t* cstart = reinterpret_cast<uint32_t*>(cbox + 2 * nch_cap);
    uint32_t* cpre = cstart + 128;
    uint32_t* cinv = cpre + 129;
    __shared__ uint32_t s_nv, s_tot, s_wsum[4];
    __shared__ float4 s_lo, s_hi;
    const CandTables tabs{cstart, cpre, cinv};

    const uint32_t nb = min(ctr->n_band, a.cap);
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t ngroups = (a.sp.res[0] + 1) * (a.sp.res[1] + 1) * (a.sp.res[2] + 1);

    for (uint32_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
        if (!a.gkey[g]) continue;  // uniform across the block
        int c[3], lo[3], hi[3];
        if (!group_box(g, a.sp, a.sc, ratio, c, lo, hi)) continue;
        const int nx = hi[0] - lo[0], ny = hi[1] - lo[1], nz = hi[2] - lo[2];
        const int nbox = nx * ny * nz;

        // 1. the group's vertices with dL/dphi != 0
        if (tid == 0) s_nv = 0;
        __syncthreads();
        for (int base = 0; base < nbox; base += kBT) {
            const int i = base + tid;
            float gv = 0.f;
            int lx = 0, ly = 0, lz = 0;
            if (i < nbox) {
                lx = i % nx;
                ly = (i / nx) % ny;
                lz = i / (nx * ny);
                const uint32_t v = lin3(lo[0] + lx, lo[1] + ly, lo[2] + lz, a.sc);
                if (band_has(a.band, v)) {
                    const uint32_t rank = band_rank(a.band, v);
                    if (rank < nb) gv = __ldg(a.gphi + rank);
                }
            }
            const bool act = gv != 0.f;
            const uint32_t m = __ballot_sync(0xffffffffu, act);
            uint32_t off = 0;
            if (lane == 0 && m) off = atomicAdd(&s_nv, __popc(m));
            off = __shfl_sync(0xffffffffu, off, 0);
            if (act) {
                const uint32_t slot = off + __popc(m & ((1u << lane) - 1u));
                if (slot < a.vlist_cap)
                    av[slot] = make_float4(vpos1(lo[0] + lx, a.sc.min[0], a.sc.cs),
                                           vpos1(lo[1] + ly, a.sc.min[1], a.sc.cs),
                                           vpos1(lo[2] + lz, a.sc.min[2], a.sc.cs), gv);
            }
        }
        __syncthreads();
        const uint32_t nv = min(s_nv, a.vlist_cap);
        if (nv == 0) continue;
        const uint32_t nch = (nv + 31) / 32;
        for (uint32_t k = tid; k < nch; k += kBT) {
            float4 l = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f), h = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
            for (uint32_t q = 32 * k; q < min(nv, 32 * k + 32); ++q) {
                const float4 v = av[q];
                l.x = fminf(l.x, v.x); l.y = fminf(l.y, v.y); l.z = fminf(l.z, v.z);
                h.x = fmaxf(h.x, v.x); h.y = fmaxf(h.y, v.y); h.z = fmaxf(h.z, v.z);
            }
            cbox[2 * k] = l;
            cbox[2 * k + 1] = h;
        }
        __syncthreads();
        if (tid == 0) {
            float4 l = cbox[0], h = cbox[1];
            for (uint32_t k = 1; k < nch; ++k) {
                const float4 kl = cbox[2 * k], kh = cbox[2 * k + 1];
                l.x = fminf(l.x, kl.x); l.y = fminf(l.y, kl.y); l.z = fminf(l.z, kl.z);
                h.x = fmaxf(h.x, kh.x); h.y = fmaxf(h.y, kh.y); h.z = fmaxf(h.z, kh.z);
            }
            s_lo = l;
            s_hi = h;
        }
        __syncthreads();
        const float4 glo = s_lo, ghi = s_hi;

        // 2. candidate cells whose reach touches the active vertices
        const float b0[3] = {glo.x, glo.y, glo.z}, b1[3] = {ghi.x, ghi.y, ghi.z};
        const uint32_t total = group_candidates(a.sp, a.ranges, a.invol, a.reach, c, b0, b1, tabs, s_wsum, &s_tot);

        // 3. one candidate per thread, gradient kept in registers
        for (uint32_t cb = 0; cb < total; cb += kBT) {
            const uint32_t j = cb + tid;
            if (j >= total) continue;
            int cell;
            const uint32_t i = candidate(j, tabs, &cell);
            const bool inv = cinv[cell] != 0;
            float4 r[4];
            load_record(a.grec, a.smoothed, a.sigma, i, inv, r);
            const float4 r0 = r[0], g0 = r[1], g1 = r[2], g2 = r[3];
            if (!(box_dist2(r0.x, r0.y, r0.z, glo, ghi) < r0.w)) continue;
            const float coef = g0.w;
            float gxs = 0.f, gys = 0.f, gzs = 0.f, sc = 0.f;
            float gg[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (uint32_t k = 0; k < nch; ++k) {
                if (!(box_dist2(r0.x, r0.y, r0.z, cbox[2 * k], cbox[2 * k + 1]) < r0.w)) continue;
                const uint32_t qe = min(nv, 32 * k + 32);
                for (uint32_t q = 32 * k; q < qe; ++q) {
                    const float4 v = av[q];
                    const float rx = r0.x - v.x, ry = r0.y - v.y, rz = r0.z - v.z;
                    const float d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                    if (!(d2 < r0.w)) continue;
                    const float tx = fmaf(g0.x, rx, fmaf(g0.y, ry, g0.z * rz));
                    const float ty = fmaf(g1.x, rx, fmaf(g1.y, ry, g1.z * rz));
                    const float tz = fmaf(g2.x, rx, fmaf(g2.y, ry, g2.z * rz));
                    const float q2 = fmaf(tx, tx, fmaf(ty, ty, tz * tz));
                    if (!(q2 < 1.0f)) continue;
                    const float u = 1.0f - q2;
                    const float A = -6.0f * v.w * coef * u * u;
                    gxs += A * (g0.x * tx + g1.x * ty + g2.x * tz);
                    gys += A * (g0.y * tx + g1.y * ty + g2.y * tz);
                    gzs += A * (g0.z * tx + g1.z * ty + g2.z * tz);
                    gg[0] += A * tx * rx; gg[1] += A * tx * ry; gg[2] += A * tx * rz;
                    gg[3] += A * ty * rx; gg[4] += A * ty * ry; gg[5] += A * ty * rz;
                    gg[6] += A * tz * rx; gg[7] += A * tz * ry; gg[8] += A * tz * rz;
                    sc += v.w * u * u * u;
                }
            }
            if (gxs != 0.f || gys != 0.f || gzs != 0.f || sc != 0.f) {
                atomicAdd(a.gsmooth + i, make_float4(gxs, gys, gzs, sc));
                if (inv) {
                    atomicAdd(a.gG + 3ull * i, make_float4(gg[0], gg[1], gg[2], 0.f));
                    atomicAdd(a.gG + 3ull * i + 1, make_float4(gg[3], gg[4], gg[5], 0.f));
                    atomicAdd(a.gG + 3ull * i + 2, make_float4(gg[6], gg[7], gg[8], 0.f));
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace

bool launch_field_aniso_backward_grouped(const KernelCtx& c, const AnisoBwdArgs& f, uint32_t ratio,
                                         const Counters* ctr)
{
    const uint32_t vcap = (ratio + 2) * (ratio + 2) * (ratio + 2);
    const size_t smem = sizeof(float4) * vcap + sizeof(float4) * 2 * ((vcap + 31) / 32) +
                        sizeof(uint32_t) * (128 + 129 + 128);
    if (smem > 200 * 1024) return false;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_field_aniso_backward_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        configured = true;
    }
    BwdGroupArgs a;
    a.sp = f.sp;
    a.sc = f.sc;
    a.band = f.band;
    a.grec = f.grec;
    a.smoothed = f.smoothed;
    a.ranges = f.ranges;
    a.invol = f.invol;
    a.reach = f.cell_rmax;
    a.gphi = f.gphi;
    a.gkey = f.gkey;
    a.gsmooth = f.gsmooth;
    a.gG = f.gG;
    a.sigma = f.sigma;
    a.cap = f.cap;
    a.vlist_cap = vcap;
    const uint64_t groups = (uint64_t)(f.sp.res[0] + 1) * (f.sp.res[1] + 1) * (f.sp.res[2] + 1);
    const unsigned grid = (unsigned)std::min<uint64_t>(
        groups, std::max<uint64_t>(1, (uint64_t)c.num_sms * 8 / std::max(1, c.grid_div)));
    k_field_aniso_backward_grouped<<<grid, kBT, smem, c.stream>>>(a, ratio, ctr);
    ++g_launches;
    return true;
}

bool launch_field_aniso_grouped(const KernelCtx& c, const AnisoFieldArgs& f, const BandView& band, uint32_t ratio,
                                Counters* ctr)
{
    // the group's index box is at most (ratio + 2)^3 vertices
    const uint32_t vcap = (ratio + 2) * (ratio + 2) * (ratio + 2);
    const size_t smem = sizeof(float4) * 4 * kChunk + sizeof(float4) * 2 * ((vcap + 31) / 32) +
                        3 * sizeof(uint32_t) * vcap + sizeof(uint16_t) * kWarps * kChunk +
                        sizeof(uint32_t) * (128 + 129 + 128);
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
    const unsigned grid = (unsigned)std::min<uint64_t>(
        groups, std::max<uint64_t>(1, (uint64_t)c.num_sms * 8 / std::max(1, c.grid_div)));
    k_field_aniso_grouped<<<grid, kBT, smem, c.stream>>>(a, ratio, ctr);
    ++g_launches;
    return true;
}

}  // namespace fsr
