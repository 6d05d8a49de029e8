// The reference's kernel-level ABI (include/fsr_compat.h), implemented on
// the reference's dense buffers with this library's kernels.
//
// Every launcher reproduces the thread-domain semantics of its reference
// kernel: the logical thread count is the product of the caller's grid and
// block dimensions, threads are numbered as getThreadIdGlobal numbers them
// (ReconstructionCUDA.cu:40-47), and each kernel here walks
// min(thread count, the reference's own bound) work items with a
// grid-stride loop.  Decision arithmetic (cell indices, vertex positions,
// band and neighbour tests, the smoothing mean, the colour field) uses the
// reference's FP32 operations without contraction, as the native kernels
// do.  Like the reference, each launcher synchronises the device before it
// returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../../include/fsr_compat.h"
#include "cov_solver.cuh"
#include "fsr_common.cuh"
#include "fsr_internal.h"
#include "kernels.h"
#include "primitives.h"

namespace fsr {
namespace compat {
namespace {

__constant__ McConst c_tables;

constexpr int kT = 256;
constexpr int kMaxDevices = 64;

std::mutex g_mutex;
bool g_tables_ready[kMaxDevices] = {};

struct Pool {
    DevBuf k0, v0, k1, v1, radix, scan, tmp_pos, tmp_den, ctr;
};
Pool g_pool[kMaxDevices];

int current_device()
{
    int d = 0;
    cudaGetDevice(&d);
    return (d >= 0 && d < kMaxDevices) ? d : 0;
}

void ensure_tables()
{
    const int d = current_device();
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_tables_ready[d]) return;
    McConst h;
    for (int i = 0; i < 256; ++i) {
        h.tri[i] = mc::kTriPacked[i];
        h.eflags[i] = mc::kDerived.eflags[i];
        h.nverts[i] = mc::kDerived.nverts[i];
    }
    if (cudaMemcpyToSymbol(c_tables, &h, sizeof(h)) == cudaSuccess) g_tables_ready[d] = true;
}

inline uint64_t domain(dim3 g, dim3 b)
{
    return (uint64_t)g.x * g.y * g.z * (uint64_t)b.x * b.y * b.z;
}

inline unsigned blocks(uint64_t n)
{
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + kT - 1) / kT, 65535ull * 16));
}

inline void finish()
{
    cudaDeviceSynchronize();
}

// ---- helpers on the reference's types
__device__ __forceinline__ Grid to_grid(const GridInfo& g)
{
    Grid r;
    r.min[0] = g.minPos.x;
    r.min[1] = g.minPos.y;
    r.min[2] = g.minPos.z;
    r.cs = g.cellSize;
    r.res[0] = g.resolution.x;
    r.res[1] = g.resolution.y;
    r.res[2] = g.resolution.z;
    r.pad = 0;
    return r;
}

__device__ __forceinline__ Grid res_grid(uint3 res)
{
    Grid r{};
    r.res[0] = res.x;
    r.res[1] = res.y;
    r.res[2] = res.z;
    return r;
}

#define GRID_STRIDE(i, n) for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
                               i += (uint64_t)gridDim.x * blockDim.x)

// ---- surface particles (cu:70-120, 466-551)
__global__ void k_surface(uint64_t n, DensityGrid flag, IsSurfaceGrid sflag, ParticleIndexRangeGrid ranges,
                          NumInvolveParticlesGrid ninv, int involve)
{
    const Grid fr = res_grid(flag.resolution), rr = res_grid(ranges.resolution);
    GRID_STRIDE(t, n)
    {
        uint32_t x, y, z;
        unlin3((uint32_t)t, rr, x, y, z);
        if (x >= fr.res[0] - 1 || y >= fr.res[1] - 1 || z >= fr.res[2] - 1) continue;
        if (flag.grid[t] < 1.0f) continue;
        const Window w = window((int)x, (int)y, (int)z, 1, fr);
        bool s = false;
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx)
                    if (flag.grid[lin3(xx, yy, zz, fr)] < 1.0f) s = true;
        if (!s) continue;
        const IndexRange r = ranges.grid[t];
        if (r.start != kEmpty)
            for (uint32_t i = r.start; i < r.end; ++i) sflag.grid[i] = 1;
        if (!involve) continue;
        const Window w2 = window((int)x, (int)y, (int)z, 2, rr);
        for (int zz = w2.lo[2]; zz <= w2.hi[2]; ++zz)
            for (int yy = w2.lo[1]; yy <= w2.hi[1]; ++yy)
                for (int xx = w2.lo[0]; xx <= w2.hi[0]; ++xx) {
                    const uint32_t c = lin3(xx, yy, zz, rr);
                    const IndexRange q = ranges.grid[c];
                    if (q.start == kEmpty) continue;
                    ninv.grid[c] = q.end - q.start;
                }
    }
}

// ---- band from the occupancy grid (cu:123-175)
__global__ void k_estimate_surface_vertices(uint64_t n, DensityGrid dens, IsSurfaceGrid band, uint ext, uint ratio)
{
    const Grid dr = res_grid(dens.resolution), br = res_grid(band.resolution);
    GRID_STRIDE(t, n)
    {
        uint32_t x, y, z;
        unlin3((uint32_t)t, dr, x, y, z);
        if (x >= dr.res[0] - 1 || y >= dr.res[1] - 1 || z >= dr.res[2] - 1) continue;
        uint32_t f = 0;
        for (int i = 0; i < 8; ++i) {
            const uint32_t c = lin3(x + mc::cornerDx(i), y + mc::cornerDy(i), z + mc::cornerDz(i), dr);
            if (dens.grid[c] <= 0.5f) f |= 1u << i;
        }
        if (f == 0 || f >= 255) continue;
        const int lo[3] = {(int)x * (int)ratio - (int)ext, (int)y * (int)ratio - (int)ext, (int)z * (int)ratio - (int)ext};
        const int hi[3] = {((int)x + 1) * (int)ratio + (int)ext, ((int)y + 1) * (int)ratio + (int)ext,
                           ((int)z + 1) * (int)ratio + (int)ext};
        const int l0 = clampi(lo[0], 0, br.res[0] - 1), h0 = clampi(hi[0], 0, br.res[0] - 1);
        const int l1 = clampi(lo[1], 0, br.res[1] - 1), h1 = clampi(hi[1], 0, br.res[1] - 1);
        const int l2 = clampi(lo[2], 0, br.res[2] - 1), h2 = clampi(hi[2], 0, br.res[2] - 1);
        for (int zz = l2; zz <= h2; ++zz)
            for (int yy = l1; yy <= h1; ++yy)
                for (int xx = l0; xx <= h0; ++xx) band.grid[lin3(xx, yy, zz, br)] = 1;
    }
}

// ---- compactions (cu:293-304, 367-380, 661-686)
__global__ void k_compact(uint64_t n, uint32_t* out, const uint32_t* scan, const uint32_t* flags)
{
    GRID_STRIDE(t, n)
    {
        if (flags[t] == 1) out[scan[t]] = (uint32_t)t;
    }
}

__global__ void k_compact_particles(uint64_t n, const uint32_t* ninv, const uint32_t* ninv_scan,
                                    const IndexRange* ranges, uint32_t* out)
{
    GRID_STRIDE(t, n)
    {
        if (ninv[t] == 0) continue;
        const uint32_t start = ninv_scan[t];
        const IndexRange r = ranges[t];
        for (uint32_t i = 0; i < r.end - r.start; ++i) out[start + i] = r.start + i;
    }
}

// ---- ZB05 field on the dense grid (cu:230-289, 308-324)
__global__ void k_zb05(uint64_t n, SurfaceVerticesIndexArray sv, ParticleIndexRangeGrid ranges, ParticleArray parts,
                       ScalarFieldGrid field, GridInfo spi, GridInfo sci, SimParam p)
{
    const Grid sp = to_grid(spi), sc = to_grid(sci), fr = res_grid(field.resolution), rr = res_grid(ranges.resolution);
    const float h2 = p.smoothingRadiusSq, inv_h2 = 1.0f / p.smoothingRadiusSq;
    GRID_STRIDE(t, n)
    {
        const uint32_t v = sv.grid[t];
        uint32_t x, y, z;
        unlin3(v, fr, x, y, z);
        const float vx = vpos1(x, sc.min[0], sc.cs), vy = vpos1(y, sc.min[1], sc.cs), vz = vpos1(z, sc.min[2], sc.cs);
        const Window w = window(cell1(vx, sp.min[0], sp.cs), cell1(vy, sp.min[1], sp.cs), cell1(vz, sp.min[2], sp.cs),
                                1, rr);
        float ws = 0.f, ax = 0.f, ay = 0.f, az = 0.f;
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx) {
                    const IndexRange r = ranges.grid[lin3(xx, yy, zz, rr)];
                    if (r.start == kEmpty) continue;
                    for (uint32_t i = r.start; i < r.end; ++i) {
                        const float3 q = parts.grid[i].pos;
                        const float dx = q.x - vx, dy = q.y - vy, dz = q.z - vz;
                        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        if (d2 < h2) {
                            const float u = 1.0f - d2 * inv_h2;
                            const float wt = u * u * u;
                            ws += wt;
                            ax = fmaf(dx, wt, ax);
                            ay = fmaf(dy, wt, ay);
                            az = fmaf(dz, wt, az);
                        }
                    }
                }
        if (ws > 0.f) field.grid[v].value = sqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az))) / ws - p.particleRadius;
    }
}

// ---- MC classify (cu:328-364, 974-1008)
__global__ void k_classify(uint64_t n, SurfaceVerticesIndexArray sv, ScalarFieldGrid field, IsValidSurfaceGrid valid,
                           NumVerticesGrid nverts, IsSurfaceGrid band, float iso, int with_nverts)
{
    const Grid fr = res_grid(field.resolution);
    GRID_STRIDE(t, n)
    {
        const uint32_t v = sv.grid[t];
        uint32_t x, y, z;
        unlin3(v, fr, x, y, z);
        if (x >= fr.res[0] - 1 || y >= fr.res[1] - 1 || z >= fr.res[2] - 1) continue;
        uint32_t f = 0;
        bool all = true;
        for (int i = 0; i < 8; ++i) {
            const uint32_t c = lin3(x + mc::cornerDx(i), y + mc::cornerDy(i), z + mc::cornerDz(i), fr);
            if (field.grid[c].value <= iso) f |= 1u << i;
            all = all && band.grid[c] != 0;
        }
        const uint32_t nv = all ? c_tables.nverts[f] : 0u;
        valid.grid[t] = nv > 0 ? 1u : 0u;
        if (with_nverts) nverts.grid[t] = nv;
    }
}

__device__ __forceinline__ float cvalue(const ScalarFieldGrid& g, const Grid& fr, int x, int y, int z)
{
    if (x < 0 || y < 0 || z < 0 || (uint32_t)x >= fr.res[0] || (uint32_t)y >= fr.res[1] || (uint32_t)z >= fr.res[2])
        return 0.f;
    return g.grid[lin3(x, y, z, fr)].value;
}

// ---- MC generation (cu:383-463)
__global__ void k_generate(uint64_t n, SurfaceVerticesIndexArray sv, ValidSurfaceIndexArray vidx, GridInfo sci,
                           NumVerticesGrid nvscan, ScalarFieldGrid field, Float3Grid pos, Float3Grid nrm, float iso)
{
    const Grid fr = res_grid(field.resolution), sc = to_grid(sci);
    const float sgn = iso < 0.0f ? -1.0f : 1.0f;
    GRID_STRIDE(t, n)
    {
        const uint32_t s = vidx.grid[t];
        uint32_t x, y, z;
        unlin3(sv.grid[s], fr, x, y, z);
        float val[8], cp[8][3], cn[8][3];
        uint32_t f = 0;
        for (int i = 0; i < 8; ++i) {
            const int cx = (int)x + mc::cornerDx(i), cy = (int)y + mc::cornerDy(i), cz = (int)z + mc::cornerDz(i);
            val[i] = cvalue(field, fr, cx, cy, cz);
            if (val[i] <= iso) f |= 1u << i;
            cp[i][0] = vpos1(cx, sc.min[0], sc.cs);
            cp[i][1] = vpos1(cy, sc.min[1], sc.cs);
            cp[i][2] = vpos1(cz, sc.min[2], sc.cs);
            float nx = cvalue(field, fr, cx - 1, cy, cz) - cvalue(field, fr, cx + 1, cy, cz);
            float ny = cvalue(field, fr, cx, cy - 1, cz) - cvalue(field, fr, cx, cy + 1, cz);
            float nz = cvalue(field, fr, cx, cy, cz - 1) - cvalue(field, fr, cx, cy, cz + 1);
            const float inv = rsqrtf(fmaf(nx, nx, fmaf(ny, ny, nz * nz)));
            cn[i][0] = nx * inv;
            cn[i][1] = ny * inv;
            cn[i][2] = nz * inv;
        }
        const uint32_t ef = c_tables.eflags[f], nv = c_tables.nverts[f];
        float ip[12][3], in[12][3];
        for (int e = 0; e < 12; ++e) {
            if (!(ef & (1u << e))) continue;
            const int a = mc::edgeA(e), b = mc::edgeB(e);
            const float d = val[b] - val[a];
            const float lf = (d > -1.0e-7f && d < 1.0e-7f) ? 0.5f : (iso - val[a]) / d;
            for (int k = 0; k < 3; ++k) {
                ip[e][k] = fmaf(lf, cp[b][k] - cp[a][k], cp[a][k]);
                in[e][k] = fmaf(lf, cn[b][k] - cn[a][k], cn[a][k]);
            }
            const float inv = rsqrtf(fmaf(in[e][0], in[e][0], fmaf(in[e][1], in[e][1], in[e][2] * in[e][2])));
            for (int k = 0; k < 3; ++k) in[e][k] *= sgn * inv;
        }
        const uint64_t tri = c_tables.tri[f];
        const uint32_t base = nvscan.grid[s];
        for (uint32_t k = 0; k < nv; ++k) {
            const int e = (int)((tri >> (4u * k)) & 0xFu);
            pos.grid[base + k] = make_float3(ip[e][0], ip[e][1], ip[e][2]);
            nrm.grid[base + k] = make_float3(in[e][0], in[e][1], in[e][2]);
        }
    }
}

// ---- narrow band (cu:554-595)
__global__ void k_band(uint64_t n, GridInfo sci, ParticleArray parts, IsSurfaceGrid sflag, IsSurfaceGrid band,
                       float thr)
{
    const Grid sc = to_grid(sci), br = res_grid(band.resolution);
    GRID_STRIDE(t, n)
    {
        if (sflag.grid[t] == 0) continue;
        const float3 p = parts.grid[t].pos;
        const Window w = window(cell1(p.x, sc.min[0], sc.cs), cell1(p.y, sc.min[1], sc.cs), cell1(p.z, sc.min[2], sc.cs),
                                3, br);
        for (int z = w.lo[2]; z <= w.hi[2]; ++z)
            for (int y = w.lo[1]; y <= w.hi[1]; ++y)
                for (int x = w.lo[0]; x < w.hi[0]; ++x) {
                    const float dx = __fsub_rn(vpos1(x, sc.min[0], sc.cs), p.x);
                    const float dy = __fsub_rn(vpos1(y, sc.min[1], sc.cs), p.y);
                    const float dz = __fsub_rn(vpos1(z, sc.min[2], sc.cs), p.z);
                    if (__fsqrt_rn(dot3_rn(dx, dy, dz)) <= thr) band.grid[lin3(x, y, z, br)] = 1;
                }
    }
}

// ---- smoothing (cu:598-658), exact FP32 in the reference's order
__global__ void k_smooth_dense(uint64_t n, SimParam p, ParticleArray parts, ParticleArray mean, ParticleArray smoothed,
                               ParticleIndexRangeGrid ranges, GridInfo spi, float one_minus_lambda)
{
    const Grid sp = to_grid(spi), rr = res_grid(ranges.resolution);
    const float R = p.anisotropicRadius, lam = p.lambdaForSmoothed;
    GRID_STRIDE(t, n)
    {
        const float3 q = parts.grid[t].pos;
        const Window w = window(cell1(q.x, sp.min[0], sp.cs), cell1(q.y, sp.min[1], sp.cs), cell1(q.z, sp.min[2], sp.cs),
                                2, rr);
        float ws = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx) {
                    const IndexRange r = ranges.grid[lin3(xx, yy, zz, rr)];
                    if (r.start == kEmpty) continue;
                    for (uint32_t i = r.start; i < r.end; ++i) {
                        const float3 o = parts.grid[i].pos;
                        const float d = __fsqrt_rn(dot3_rn(__fsub_rn(q.x, o.x), __fsub_rn(q.y, o.y), __fsub_rn(q.z, o.z)));
                        float wt = 0.f;
                        if (d < R) {
                            const float s = __fdiv_rn(d, R);
                            wt = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(s, s), s));
                        }
                        ws = __fadd_rn(ws, wt);
                        mx = __fadd_rn(mx, __fmul_rn(o.x, wt));
                        my = __fadd_rn(my, __fmul_rn(o.y, wt));
                        mz = __fadd_rn(mz, __fmul_rn(o.z, wt));
                    }
                }
        if (ws > 0.f) {
            mx = __fdiv_rn(mx, ws);
            my = __fdiv_rn(my, ws);
            mz = __fdiv_rn(mz, ws);
            mean.grid[t].pos = make_float3(mx, my, mz);
            smoothed.grid[t].pos = make_float3(__fadd_rn(__fmul_rn(one_minus_lambda, q.x), __fmul_rn(lam, mx)),
                                               __fadd_rn(__fmul_rn(one_minus_lambda, q.y), __fmul_rn(lam, my)),
                                               __fadd_rn(__fmul_rn(one_minus_lambda, q.z), __fmul_rn(lam, mz)));
        }
    }
}

// ---- covariance and G (cu:689-827), shared solver with the native kernel
__global__ void k_cov_dense(uint64_t n, SimParam p, GridInfo spi, ParticleArray mean, ParticleArray parts,
                            ParticleIndexRangeGrid ranges, SurfaceParticlesIndexArray idx, MatrixArray mats)
{
    const Grid sp = to_grid(spi), rr = res_grid(ranges.resolution);
    const float R = p.anisotropicRadius;
    GRID_STRIDE(t, n)
    {
        const uint32_t pi = idx.grid[t];
        const float3 q = parts.grid[pi].pos;
        const float3 m = mean.grid[pi].pos;
        const Window w = window(cell1(q.x, sp.min[0], sp.cs), cell1(q.y, sp.min[1], sp.cs), cell1(q.z, sp.min[2], sp.cs),
                                2, rr);
        CovAccum acc;
        uint32_t nn = 0;
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx) {
                    const IndexRange r = ranges.grid[lin3(xx, yy, zz, rr)];
                    if (r.start == kEmpty) continue;
                    for (uint32_t i = r.start; i < r.end; ++i) {
                        const float3 o = parts.grid[i].pos;
                        const float vx = __fsub_rn(o.x, m.x), vy = __fsub_rn(o.y, m.y), vz = __fsub_rn(o.z, m.z);
                        const float d = __fsqrt_rn(dot3_rn(vx, vy, vz));
                        if (d <= R) ++nn;
                        if (d < R) acc.add(vx, vy, vz, __fdiv_rn(d, R));
                    }
                }
        float G[9];
        covariance_to_G(acc, nn, p.minNumNeighbors, p.smoothingRadius, p.smoothingRadiusSq, p.smoothingRadiusInv, G,
                        nullptr);
        MatrixValue o;
        o.a11 = G[0]; o.a12 = G[1]; o.a13 = G[2];
        o.a21 = G[3]; o.a22 = G[4]; o.a23 = G[5];
        o.a31 = G[6]; o.a32 = G[7]; o.a33 = G[8];
        mats.grid[t] = o;
    }
}

// ---- anisotropic field (cu:830-906)
__global__ void k_aniso_dense(uint64_t n, SimParam p, GridInfo sci, GridInfo spi, MatrixArray mats,
                              ParticleArray smoothed, ScalarFieldGrid dens, ParticleIndexRangeGrid ranges,
                              SurfaceVerticesIndexArray sv, NumInvolveParticlesGrid ninv, NumInvolveParticlesGrid ninv_scan,
                              ScalarFieldGrid field, float sigma)
{
    const Grid sp = to_grid(spi), sc = to_grid(sci), fr = res_grid(field.resolution), rr = res_grid(ranges.resolution);
    GRID_STRIDE(t, n)
    {
        const uint32_t v = sv.grid[t];
        uint32_t x, y, z;
        unlin3(v, fr, x, y, z);
        const float vx = vpos1(x, sc.min[0], sc.cs), vy = vpos1(y, sc.min[1], sc.cs), vz = vpos1(z, sc.min[2], sc.cs);
        const Window w = window(cell1(vx, sp.min[0], sp.cs), cell1(vy, sp.min[1], sp.cs), cell1(vz, sp.min[2], sp.cs),
                                2, rr);
        float sum = 0.f;
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx) {
                    const uint32_t c = lin3(xx, yy, zz, rr);
                    const IndexRange r = ranges.grid[c];
                    if (ninv.grid[c] > 0) {
                        const uint32_t g0 = ninv_scan.grid[c];
                        for (uint32_t i = 0; i < r.end - r.start; ++i) {
                            const MatrixValue g = mats.grid[g0 + i];
                            const float3 s = smoothed.grid[r.start + i].pos;
                            const float rx = s.x - vx, ry = s.y - vy, rz = s.z - vz;
                            const float tx = fmaf(g.a11, rx, fmaf(g.a12, ry, g.a13 * rz));
                            const float ty = fmaf(g.a21, rx, fmaf(g.a22, ry, g.a23 * rz));
                            const float tz = fmaf(g.a31, rx, fmaf(g.a32, ry, g.a33 * rz));
                            const float q2 = fmaf(tx, tx, fmaf(ty, ty, tz * tz));
                            if (q2 < 1.0f) {
                                const float det = g.a11 * g.a22 * g.a33 + g.a12 * g.a23 * g.a31 + g.a13 * g.a21 * g.a32 -
                                                  g.a11 * g.a23 * g.a32 - g.a12 * g.a21 * g.a33 - g.a13 * g.a22 * g.a31;
                                const float u = 1.0f - q2;
                                sum = fmaf(p.particleMass / dens.grid[r.start + i].value * sigma * det, u * u * u, sum);
                            }
                        }
                    } else {
                        if (r.start == kEmpty) continue;
                        for (uint32_t i = r.start; i < r.end; ++i) {
                            const float3 s = smoothed.grid[i].pos;
                            const float rx = s.x - vx, ry = s.y - vy, rz = s.z - vz;
                            const float d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                            if (d2 < 1.0f) {
                                const float u = 1.0f - d2;
                                sum = fmaf(p.particleMass / dens.grid[i].value * sigma, u * u * u, sum);
                            }
                        }
                    }
                }
        field.grid[v].value = sum - 0.5f;
    }
}

// ---- Akinci12 colour field (cu:909-971), exact as the native kernel
__global__ void k_colorfield_dense(uint64_t n, SimParam p, ParticleArray parts, ScalarFieldGrid dens,
                                   ParticleIndexRangeGrid ranges, GridInfo spi, IsSurfaceGrid sflag, double k_spiky)
{
    const Grid sp = to_grid(spi), rr = res_grid(ranges.resolution);
    const float h = p.smoothingRadius, mass = p.particleMass;
    GRID_STRIDE(t, n)
    {
        const float3 q = parts.grid[t].pos;
        const Window w = window(cell1(q.x, sp.min[0], sp.cs), cell1(q.y, sp.min[1], sp.cs), cell1(q.z, sp.min[2], sp.cs),
                                1, rr);
        uint32_t nn = 0;
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx) {
                    const IndexRange r = ranges.grid[lin3(xx, yy, zz, rr)];
                    if (r.start == kEmpty) continue;
                    for (uint32_t i = r.start; i < r.end; ++i) {
                        const float3 o = parts.grid[i].pos;
                        float rx = __fsub_rn(q.x, o.x), ry = __fsub_rn(q.y, o.y), rz = __fsub_rn(q.z, o.z);
                        const float d2 = dot3_rn(rx, ry, rz);
                        if (!(d2 > 0.0f)) continue;
                        ++nn;
                        const float d = __fsqrt_rn(d2);
                        float grad = 0.0f;
                        if (!(d >= h)) {
                            const float x = __double2float_rn(__dsub_rn(1.0, (double)__fdiv_rn(d, h)));
                            grad = __double2float_rn(__dmul_rn(__dmul_rn(k_spiky, (double)x), (double)x));
                        }
                        const float inv = __fdiv_rn(1.0f, __fsqrt_rn(d2));
                        const float coef = __fmul_rn(__fdiv_rn(mass, dens.grid[i].value), grad);
                        sx = __fadd_rn(sx, __fmul_rn(coef, __fmul_rn(rx, inv)));
                        sy = __fadd_rn(sy, __fmul_rn(coef, __fmul_rn(ry, inv)));
                        sz = __fadd_rn(sz, __fmul_rn(coef, __fmul_rn(rz, inv)));
                    }
                }
        if (nn < 25u || __fsqrt_rn(dot3_rn(sx, sy, sz)) > 3.0f) sflag.grid[t] = 1;
    }
}

// ---- spatial grid building (cu:1379-1481)
__global__ void k_hash_dense(uint32_t n, const float* xyz, GridInfo spi, uint32_t* keys, uint32_t* vals, float* flag,
                             uint32_t n_cells)
{
    const Grid sp = to_grid(spi);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool ok = true;
    int c[3];
    for (int a = 0; a < 3; ++a) {
        const float q = __fdiv_rn(__fsub_rn(xyz[3ull * i + a], sp.min[a]), sp.cs);
        ok = ok && (q > -1.0f) && (q < (float)sp.res[a]);
        c[a] = ok ? __float2int_rz(q) : 0;
    }
    // particles outside the grid sort behind every cell and get no range
    const uint32_t key = ok ? lin3(c[0], c[1], c[2], sp) : n_cells;
    keys[i] = key;
    vals[i] = i;
    if (ok) flag[key] = 1.0f;
}

__global__ void k_gather_inplace(uint32_t n, const uint32_t* skeys, const uint32_t* perm, const float* xyz_src,
                                 const float* den_src, float* xyz, float* den, IndexRange* ranges, uint32_t n_cells)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = skeys[k];
    if (key < n_cells) {
        if (k == 0 || skeys[k - 1] != key) ranges[key].start = k;
        if (k + 1 == n || skeys[k + 1] != key) ranges[key].end = k + 1;
    }
    const uint32_t s = perm[k];
    xyz[3ull * k] = xyz_src[3ull * s];
    xyz[3ull * k + 1] = xyz_src[3ull * s + 1];
    xyz[3ull * k + 2] = xyz_src[3ull * s + 2];
    den[k] = den_src[s];
}

}  // namespace
}  // namespace compat
}  // namespace fsr

using namespace fsr;
using namespace fsr::compat;

extern "C" void bindTextures(uint* d_edgeTable, int* d_edgeIndicesOfTriangleTable, uint* d_numVerticesTable,
                             uint* d_vertexIndicesOfEdgeTable)
{
    (void)d_edgeTable;
    (void)d_edgeIndicesOfTriangleTable;
    (void)d_numVerticesTable;
    (void)d_vertexIndicesOfEdgeTable;
    ensure_tables();
}

extern "C" void launchExtractionOfSurfaceParticles(dim3 g, dim3 b, SimParam simParam, DensityGrid flagGrid,
                                                   IsSurfaceGrid sflag, ParticleIndexRangeGrid ranges)
{
    (void)simParam;
    const uint64_t n = std::min<uint64_t>(domain(g, b), ranges.size);
    k_surface<<<blocks(n), kT>>>(n, flagGrid, sflag, ranges, NumInvolveParticlesGrid{}, 0);
    finish();
}

extern "C" void launchEstimateSurfaceVertices(dim3 g, dim3 b, DensityGrid densityGrid, IsSurfaceGrid isSurfaceGrid,
                                              uint scSearchExt, SimParam params)
{
    const uint64_t n = std::min<uint64_t>(domain(g, b), densityGrid.size);
    k_estimate_surface_vertices<<<blocks(n), kT>>>(n, densityGrid, isSurfaceGrid, scSearchExt,
                                                   params.scSpGridResRatio);
    finish();
}

extern "C" void launchCompactSurfaceVertex(dim3 g, dim3 b, SurfaceVerticesIndexArray sv, IsSurfaceGrid scan,
                                           IsSurfaceGrid flags, SimParam params)
{
    (void)params;
    const uint64_t n = std::min<uint64_t>(domain(g, b), scan.size);
    k_compact<<<blocks(n), kT>>>(n, sv.grid, scan.grid, flags.grid);
    finish();
}

extern "C" void launchUpdateScalarGridValuesCompacted(dim3 g, dim3 b, SurfaceVerticesIndexArray sv, uint numSV,
                                                      ParticleIndexRangeGrid ranges, ParticleArray parts,
                                                      ScalarFieldGrid field, GridInfo spi, GridInfo sci, SimParam p)
{
    const uint64_t n = std::min<uint64_t>(std::min<uint64_t>(domain(g, b), sv.size), numSV);
    k_zb05<<<blocks(n), kT>>>(n, sv, ranges, parts, field, spi, sci, p);
    finish();
}

extern "C" void launchDetectValidSurfaceCubes(dim3 g, dim3 b, SurfaceVerticesIndexArray sv, uint numSV,
                                              ScalarFieldGrid vGrid, IsValidSurfaceGrid valid, NumVerticesGrid nverts,
                                              IsSurfaceGrid band, SimParam p)
{
    ensure_tables();
    const uint64_t n = std::min<uint64_t>(std::min<uint64_t>(domain(g, b), sv.size), numSV);
    k_classify<<<blocks(n), kT>>>(n, sv, vGrid, valid, nverts, band, p.isoValue, 1);
    finish();
}

extern "C" void launchCompactValidSurfaceCubes(dim3 g, dim3 b, ValidSurfaceIndexArray idx, IsValidSurfaceGrid scan,
                                               IsValidSurfaceGrid valid, SimParam params)
{
    (void)params;
    const uint64_t n = std::min<uint64_t>(domain(g, b), scan.size);
    k_compact<<<blocks(n), kT>>>(n, idx.grid, scan.grid, valid.grid);
    finish();
}

extern "C" void launchGenerateTriangles(dim3 g, dim3 b, SurfaceVerticesIndexArray sv, ValidSurfaceIndexArray vidx,
                                        GridInfo sci, NumVerticesGrid nvscan, ScalarFieldGrid field, Float3Grid pos,
                                        Float3Grid nrm, SimParam p)
{
    ensure_tables();
    const uint64_t n = std::min<uint64_t>(domain(g, b), vidx.size);
    k_generate<<<blocks(n), kT>>>(n, sv, vidx, sci, nvscan, field, pos, nrm, p.isoValue);
    finish();
}

extern "C" uint launchThrustExclusivePrefixSumScan(uint* output, uint* input, uint numElements)
{
    if (numElements == 0) return 0;
    const int d = current_device();
    Pool& pl = g_pool[d];
    uint32_t last_in = 0, last_out = 0;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (pl.scan.ensure(4 * scan_scratch_words(numElements)) != cudaSuccess) return 0;
        // the input may alias the output: keep its last element first
        cudaMemcpy(&last_in, input + numElements - 1, 4, cudaMemcpyDeviceToHost);
        scan_u32(input, output, numElements, nullptr, numElements, nullptr, ScanInput::kValue,
                 (uint32_t*)pl.scan.ptr, 0);
        cudaMemcpy(&last_out, output + numElements - 1, 4, cudaMemcpyDeviceToHost);
    }
    return last_in + last_out;
}

extern "C" void launchExtractionOfSurfaceAndInvolveParticles(dim3 g, dim3 b, SimParam simParam, DensityGrid flagGrid,
                                                             NumInvolveParticlesGrid ninv, IsSurfaceGrid sflag,
                                                             ParticleIndexRangeGrid ranges)
{
    (void)simParam;
    const uint64_t n = std::min<uint64_t>(domain(g, b), ranges.size);
    k_surface<<<blocks(n), kT>>>(n, flagGrid, sflag, ranges, ninv, 1);
    finish();
}

extern "C" void launchEstimationOfSurfaceVertices(dim3 g, dim3 b, SimParam p, GridInfo sci, ParticleArray parts,
                                                  IsSurfaceGrid sflag, ParticleIndexRangeGrid ranges,
                                                  IsSurfaceGrid band)
{
    (void)ranges;
    const uint64_t n = std::min<uint64_t>(domain(g, b), sflag.size);
    k_band<<<blocks(n), kT>>>(n, sci, parts, sflag, band, band_threshold(p.smoothingRadius));
    finish();
}

extern "C" void launchCalculationOfMeanAndSmoothParticles(dim3 g, dim3 b, SimParam p, ParticleArray parts,
                                                          ParticleArray mean, ParticleArray smoothed,
                                                          ParticleIndexRangeGrid ranges, GridInfo spi)
{
    const uint64_t n = std::min<uint64_t>(domain(g, b), parts.size);
    k_smooth_dense<<<blocks(n), kT>>>(n, p, parts, mean, smoothed, ranges, spi,
                                      (float)(1.0 - (double)p.lambdaForSmoothed));
    finish();
}

extern "C" void launchCompactationOfSurfaceVerticesAndParticles(dim3 g, dim3 b, SimParam simParam, IsSurfaceGrid band,
                                                                IsSurfaceGrid bandScan, NumInvolveParticlesGrid ninv,
                                                                NumInvolveParticlesGrid ninvScan,
                                                                ParticleIndexRangeGrid ranges,
                                                                SurfaceVerticesIndexArray sv,
                                                                SurfaceParticlesIndexArray sp)
{
    (void)simParam;
    const uint64_t d = domain(g, b);
    const uint64_t n1 = std::min<uint64_t>(d, bandScan.size);
    const uint64_t n2 = std::min<uint64_t>(d, ninvScan.size);
    k_compact<<<blocks(n1), kT>>>(n1, sv.grid, bandScan.grid, band.grid);
    k_compact_particles<<<blocks(n2), kT>>>(n2, ninv.grid, ninvScan.grid, ranges.grid, sp.grid);
    finish();
}

extern "C" void launchCalculationOfTransformMatricesForParticles(dim3 g, dim3 b, SimParam p, GridInfo spi,
                                                                 ParticleArray mean, ParticleArray parts,
                                                                 ParticleIndexRangeGrid ranges,
                                                                 SurfaceParticlesIndexArray idx, MatrixArray mats)
{
    const uint64_t n = std::min<uint64_t>(domain(g, b), idx.size);
    k_cov_dense<<<blocks(n), kT>>>(n, p, spi, mean, parts, ranges, idx, mats);
    finish();
}

extern "C" void launchComputationOfScalarFieldGrid(dim3 g, dim3 b, SimParam p, uint numSV, GridInfo sci, GridInfo spi,
                                                   MatrixArray mats, ParticleArray smoothed, ScalarFieldGrid dens,
                                                   ParticleIndexRangeGrid ranges, SurfaceVerticesIndexArray sv,
                                                   NumInvolveParticlesGrid ninv, NumInvolveParticlesGrid ninvScan,
                                                   ScalarFieldGrid field)
{
    const uint64_t n = std::min<uint64_t>(std::min<uint64_t>(domain(g, b), sv.size), numSV);
    k_aniso_dense<<<blocks(n), kT>>>(n, p, sci, spi, mats, smoothed, dens, ranges, sv, ninv, ninvScan, field,
                                     315.0f / (64.0f * 3.1415926535898f));
    finish();
}

extern "C" void launchExtractionOfSurfaceParticlesForAkinci(dim3 g, dim3 b, SimParam p, ParticleArray parts,
                                                            ScalarFieldGrid dens, ParticleIndexRangeGrid ranges,
                                                            GridInfo spi, IsSurfaceGrid sflag)
{
    const uint64_t n = std::min<uint64_t>(domain(g, b), parts.size);
    const double k = -45.0 / (3.1415926535 * (double)p.smoothingRadiusSq * (double)p.smoothingRadiusSq);
    k_colorfield_dense<<<blocks(n), kT>>>(n, p, parts, dens, ranges, spi, sflag, k);
    finish();
}

extern "C" void launchDetectionOfValidSurfaceCubesForAkinci(dim3 g, dim3 b, SurfaceVerticesIndexArray sv, uint numSV,
                                                            ScalarFieldGrid vGrid, IsValidSurfaceGrid valid,
                                                            IsSurfaceGrid band, SimParam p)
{
    ensure_tables();
    const uint64_t n = std::min<uint64_t>(std::min<uint64_t>(domain(g, b), sv.size), numSV);
    k_classify<<<blocks(n), kT>>>(n, sv, vGrid, valid, NumVerticesGrid{}, band, p.isoValue, 0);
    finish();
}

extern "C" void launchSpatialGridBuilding(ParticleArray parts, ScalarFieldGrid dens, uint n,
                                          ParticleIndexRangeGrid ranges, DensityGrid flag, GridInfo spi)
{
    if (n == 0) return;
    const uint64_t C = (uint64_t)spi.resolution.x * spi.resolution.y * spi.resolution.z;
    const int d = current_device();
    Pool& pl = g_pool[d];
    std::lock_guard<std::mutex> lock(g_mutex);
    if (pl.k0.ensure(4ull * n) || pl.v0.ensure(4ull * n) || pl.k1.ensure(4ull * n) || pl.v1.ensure(4ull * n) ||
        pl.radix.ensure(4ull * radix_scratch_words(n)) || pl.tmp_pos.ensure(12ull * n) || pl.tmp_den.ensure(4ull * n))
        return;
    uint32_t* k0 = (uint32_t*)pl.k0.ptr;
    uint32_t* v0 = (uint32_t*)pl.v0.ptr;
    uint32_t* k1 = (uint32_t*)pl.k1.ptr;
    uint32_t* v1 = (uint32_t*)pl.v1.ptr;
    k_hash_dense<<<(n + 255) / 256, 256>>>(n, (const float*)parts.grid, spi, k0, v0, (float*)flag.grid, (uint32_t)C);
    cudaError_t e = cudaSuccess;
    const int which = radix_sort_pairs(k0, v0, k1, v1, n, bits_for(C + 1), (uint32_t*)pl.radix.ptr, 0, &e);
    // sort in place: stage the inputs, then gather back into the caller's arrays
    cudaMemcpyAsync(pl.tmp_pos.ptr, parts.grid, 12ull * n, cudaMemcpyDeviceToDevice, 0);
    cudaMemcpyAsync(pl.tmp_den.ptr, dens.grid, 4ull * n, cudaMemcpyDeviceToDevice, 0);
    cudaMemsetAsync(ranges.grid, 0xFF, ranges.size * sizeof(IndexRange), 0);
    k_gather_inplace<<<(n + 255) / 256, 256>>>(n, which ? k1 : k0, which ? v1 : v0, (const float*)pl.tmp_pos.ptr,
                                               (const float*)pl.tmp_den.ptr, (float*)parts.grid, (float*)dens.grid,
                                               ranges.grid, (uint32_t)C);
    finish();
}
