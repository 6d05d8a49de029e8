// Per-frame kernels of the reconstruction path.  Each kernel names the
// reference kernel it replaces (ReconstructionCUDA.cu, "cu").
#include "kernels.h"
#include "primitives.h"
#include "cov_solver.cuh"

#include <algorithm>
#include <cmath>

namespace fsr {

__constant__ McConst c_mc;
thread_local uint64_t g_launches = 0;

void upload_mc_tables(cudaStream_t s)
{
    McConst h;
    for (int i = 0; i < 256; ++i) {
        h.tri[i] = mc::kTriPacked[i];
        h.eflags[i] = mc::kDerived.eflags[i];
        h.nverts[i] = mc::kDerived.nverts[i];
    }
    cudaMemcpyToSymbolAsync(c_mc, &h, sizeof(h), 0, cudaMemcpyHostToDevice, s);
}

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(uint64_t n, int threads = kThreads)
{
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + threads - 1) / threads, 0x7fffffffULL));
}

// threads per block of the per-item and warp-staged kernels: the context's
// block shape (a multiple of 32 up to kThreads, which their per-warp shared
// arrays are sized for)
inline int bs(const KernelCtx& c) { return (c.block >= 32 && c.block <= kThreads && c.block % 32 == 0) ? c.block : kThreads; }

// grid for grid-stride kernels whose length is read on the device
inline unsigned persistent_blocks(const KernelCtx& c, uint64_t cap, int per_sm = 8)
{
    const uint64_t want = (cap + bs(c) - 1) / bs(c);
    // per_sm counts blocks of kThreads threads: smaller blocks get proportionally more
    per_sm = per_sm * (kThreads / bs(c));
    const uint64_t most = std::max<uint64_t>(1, (uint64_t)c.num_sms * per_sm / std::max(1, c.grid_div));
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, most));
}

__device__ __forceinline__ void warp_count(uint32_t* counter, bool pred)
{
    const uint32_t m = __ballot_sync(__activemask(), pred);
    if (pred && (threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(counter, __popc(m));
}

// ------------------------------------------------------------ hashing
// calcParticlesHashKernel (cu:1379-1396) plus the bounds check the
// reference lacks (cu:1391-1395 writes out of bounds for such particles).
__global__ void k_hash(const float* __restrict__ xyz, uint32_t n, Grid sp, uint32_t* __restrict__ keys,
                       uint32_t* __restrict__ vals, Counters* ctr)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float p[3] = {xyz[3ull * i], xyz[3ull * i + 1], xyz[3ull * i + 2]};
    int c[3];
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float q = __fdiv_rn(__fsub_rn(p[a], sp.min[a]), sp.cs);
        ok = ok && (q > -1.0f) && (q < (float)sp.res[a]);  // NaN fails too
        c[a] = ok ? __float2int_rz(q) : 0;
    }
    keys[i] = ok ? lin3((uint32_t)c[0], (uint32_t)c[1], (uint32_t)c[2], sp) : 0u;
    vals[i] = i;
    if (!ok) atomicAdd(&ctr->out_of_grid, 1u);
}

// findCellRangeKernel (cu:1399-1435) fused with the gather of the sorted
// particles (the reference sorts positions and densities in place,
// cu:1461-1466) into one float4 per particle.
__global__ void k_ranges_gather(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
                                uint32_t n, const float* __restrict__ xyz, const float* __restrict__ dens,
                                float4* __restrict__ sorted, uint2* __restrict__ ranges,
                                uint8_t* __restrict__ occ)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = skeys[k];
    const uint32_t prev = k > 0 ? skeys[k - 1] : kEmpty;
    const uint32_t next = k + 1 < n ? skeys[k + 1] : kEmpty;
    if (key != prev) {
        ranges[key].x = k;
        occ[key] = 1;
    }
    if (key != next) ranges[key].y = k + 1;
    const uint32_t s = perm[k];
    // without densities (computed later by k_density) w is left at 0
    sorted[k] = make_float4(xyz[3ull * s], xyz[3ull * s + 1], xyz[3ull * s + 2], dens ? dens[s] : 0.0f);
}

// SPH density of each sorted particle, for frames without a density column
// (the reference's .xyz files carry the simulator's densities and the
// reference computes none): rho_i = m sigma / h^3 sum_j (1 - |x_i - x_j|^2 /
// h^2)^3 over the particles within h, i itself included, sigma = 315 /
// (64 pi) - the poly6 kernel with the normalisation of the reference's own
// field kernel (anisotropicW, cuh:294-310, at G = I / h).  Each particle's
// sum runs over its window's cells in order, so results are deterministic.
__global__ void __launch_bounds__(kThreads) k_density(const float4* __restrict__ sorted, uint32_t n,
                                                      const uint2* __restrict__ ranges, Grid sp, int ext, float h,
                                                      float h2, float inv_h2, float scale, float* __restrict__ rho)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float4 p = sorted[t];
    const Window w = narrow(window(cell1(p.x, sp.min[0], sp.cs), cell1(p.y, sp.min[1], sp.cs),
                                   cell1(p.z, sp.min[2], sp.cs), ext, sp),
                            p.x, p.y, p.z, cull_radius(h, sp.cs), sp);
    float sum = 0.f;
    for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
        for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy) {
            // the row's cells are contiguous in the sorted array
            const uint32_t c0 = lin3(w.lo[0], yy, zz, sp);
            uint32_t beg = kEmpty, end = 0;
            for (int xx = 0; xx <= w.hi[0] - w.lo[0]; ++xx) {
                const uint2 r = __ldg(&ranges[c0 + xx]);
                if (r.x != kEmpty) {
                    beg = min(beg, r.x);
                    end = max(end, r.y);
                }
            }
            for (uint32_t i = beg; i < end; ++i) {
                const float4 q = __ldg(&sorted[i]);
                const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
                const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                if (d2 < h2) {
                    const float u = 1.0f - d2 * inv_h2;
                    sum = fmaf(u * u, u, sum);
                }
            }
        }
    rho[t] = scale * sum;
}

__global__ void k_set_density(float4* __restrict__ sorted, const float* __restrict__ rho, uint32_t n)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) sorted[t].w = rho[t];
}

// ------------------------------------------------------------ surface
// extractionOfSurfaceParticles (cu:70-120): an occupied cell with an empty
// cell in its clamped 3x3x3 neighbourhood is a surface cell; the last cell
// layer of each axis is never tested (cu:81).
__global__ void k_surface_cells(Grid sp, const uint8_t* __restrict__ occ, uint8_t* __restrict__ surf)
{
    const uint64_t C = (uint64_t)sp.res[0] * sp.res[1] * sp.res[2];
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C) return;
    uint32_t x, y, z;
    unlin3((uint32_t)t, sp, x, y, z);
    uint8_t s = 0;
    if (x < sp.res[0] - 1 && y < sp.res[1] - 1 && z < sp.res[2] - 1 && occ[t]) {
        const Window w = window((int)x, (int)y, (int)z, 1, sp);
        for (int zz = w.lo[2]; zz <= w.hi[2] && !s; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1] && !s; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx)
                    if (!occ[lin3(xx, yy, zz, sp)]) { s = 1; break; }
    }
    surf[t] = s;
}

// The involved cells of extractionOfSurfaceAndInvolveParticles (cu:519-550),
// gathered instead of scattered: an occupied cell is involved when a surface
// cell lies within +-2 cells on every axis.
__global__ void k_involved_cells(Grid sp, const uint8_t* __restrict__ occ, const uint8_t* __restrict__ surf,
                                 uint8_t* __restrict__ invol)
{
    const uint64_t C = (uint64_t)sp.res[0] * sp.res[1] * sp.res[2];
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C) return;
    uint8_t v = 0;
    if (occ[t]) {
        uint32_t x, y, z;
        unlin3((uint32_t)t, sp, x, y, z);
        const Window w = window((int)x, (int)y, (int)z, 2, sp);
        for (int zz = w.lo[2]; zz <= w.hi[2] && !v; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1] && !v; ++yy)
                for (int xx = w.lo[0]; xx <= w.hi[0]; ++xx)
                    if (surf[lin3(xx, yy, zz, sp)]) { v = 1; break; }
    }
    invol[t] = v;
}

// extractionOfSurfaceParticlesUsingColorField (cu:909-971, wSpikyGrad
// cuh:324-334).  The decision |grad c| > 3 depends on a sum, so the sum is
// taken in the reference's order with the reference's roundings (FP64 where
// the source promotes).
__global__ void __launch_bounds__(kThreads) k_colorfield(const float4* __restrict__ sorted, uint32_t n,
                                                         const uint2* __restrict__ ranges,
                                                         const uint32_t* __restrict__ skeys, Grid sp, float h,
                                                         float h_rcp, float h_lt2, double k_spiky, float khi,
                                                         float klo, float mass, uint8_t* __restrict__ psurf)
{
    __shared__ float4 s_q[kThreads];    // staged candidates, per warp
    __shared__ float s_mr[kThreads];    // their m / rho
    __shared__ uint32_t s_cx[kThreads]; // their cells' x index
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = t < n;
    if (__all_sync(0xffffffffu, !active)) return;
    const int lane = threadIdx.x & 31;
    const uint32_t wb = threadIdx.x & ~31u;
    const float4 p = active ? sorted[t] : make_float4(0.f, 0.f, 0.f, 1.f);
    const Window w = window(cell1(p.x, sp.min[0], sp.cs), cell1(p.y, sp.min[1], sp.cs),
                            cell1(p.z, sp.min[2], sp.cs), 1, sp);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    // a neighbour at squared distance 0 < d2 < h^2 (the gradient is 0 at d >= h,
    // and +0 / -0 terms leave the sums, never -0, unchanged)
    auto add = [&](float4 q, float d2, float m_rho) {
        float rx = __fsub_rn(p.x, q.x), ry = __fsub_rn(p.y, q.y), rz = __fsub_rn(p.z, q.z);
        const float d = __fsqrt_rn(d2);
        // x = float(1.0 - (double)(d / h)): the double difference of 1 and a
        // float is exact, so rounding it to float is the correctly rounded
        // FP32 difference (no FP64 work needed)
        const float x = __fsub_rn(1.0f, div_exact(d, h, h_rcp));
        // float(k x x) in double (cu:957); in FP32 when |k| is in range (khi > 0)
        const float grad = khi > 0.f ? spiky_grad(x, khi, klo, k_spiky) : spiky_grad_double(x, k_spiky);
        const float inv = __fdiv_rn(1.0f, d);
        rx = __fmul_rn(rx, inv);
        ry = __fmul_rn(ry, inv);
        rz = __fmul_rn(rz, inv);
        const float coef = __fmul_rn(m_rho, grad);
        sx = __fadd_rn(sx, __fmul_rn(coef, rx));
        sy = __fadd_rn(sy, __fmul_rn(coef, ry));
        sz = __fadd_rn(sz, __fmul_rn(coef, rz));
    };
    auto dist2 = [&](const float4& q) {
        return dot3_rn(__fsub_rn(p.x, q.x), __fsub_rn(p.y, q.y), __fsub_rn(p.z, q.z));
    };
    auto row_range = [&](int x0, int x1, int yy, int zz, uint32_t& beg, uint32_t& end, uint32_t& cnt) {
        // the particles of a row of x-adjacent cells are contiguous in sorted order
        const uint32_t c0 = lin3(x0, yy, zz, sp);
        beg = kEmpty;
        end = 0;
        cnt = 0;
        for (int xx = 0; xx <= x1 - x0; ++xx) {
            const uint2 r = __ldg(&ranges[c0 + xx]);
            if (r.x != kEmpty) {
                beg = min(beg, r.x);
                end = max(end, r.y);
                cnt += r.y - r.x;
            }
        }
    };
    // nn: the particles of the window at a distance > 0 (the reference counts
    // every particle of the 27 cells, cu:930-950) = the window's particles
    // minus those at distance 0 (the particle itself and exact duplicates)
    uint32_t nn = 0;
    int ulo[3], uhi[3];
    bool compact = true;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        ulo[ax] = (int)__reduce_min_sync(0xffffffffu, active ? (unsigned)w.lo[ax] : 0x7fffffffu);
        uhi[ax] = (int)__reduce_max_sync(0xffffffffu, active ? (unsigned)(w.hi[ax] + 1) : 0u) - 1;
        compact = compact && uhi[ax] - ulo[ax] <= 4;
    }
    if (compact) {
        // the warp walks the union of its windows; staging drops what lies
        // beyond h of every lane's particle (zero gradient, and such a
        // particle is at a distance > 0, counted through the cell counts);
        // each lane takes the staged particles of its own window in window
        // order (rows from the loop, x from the cell index)
        uint32_t in_window = 0, zeros = 0;
        if (active)
            for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
                for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy) {
                    uint32_t b, e, c;
                    row_range(w.lo[0], w.hi[0], yy, zz, b, e, c);
                    in_window += c;
                }
        const WarpBox box = warp_box(active, p.x, p.y, p.z, cull_radius(h, sp.cs));
        for (int zz = ulo[2]; zz <= uhi[2]; ++zz)
            for (int yy = ulo[1]; yy <= uhi[1]; ++yy) {
                const bool row_in = active && zz >= w.lo[2] && zz <= w.hi[2] && yy >= w.lo[1] && yy <= w.hi[1];
                if (!__any_sync(0xffffffffu, row_in)) continue;
                uint32_t beg, end, c;
                row_range(ulo[0], uhi[0], yy, zz, beg, end, c);
                for (uint32_t b = beg; b < end; b += 32) {
                    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                    bool keep = false;
                    if (b + lane < end) {
                        q = __ldg(&sorted[b + lane]);
                        keep = box.keeps(q);
                    }
                    const uint32_t mk = __ballot_sync(0xffffffffu, keep);
                    if (keep) {
                        const uint32_t slot = wb + __popc(mk & ((1u << lane) - 1u));
                        s_q[slot] = q;
                        s_mr[slot] = __fdiv_rn(mass, q.w);
                        s_cx[slot] = __ldg(&skeys[b + lane]) % sp.res[0];
                    }
                    __syncwarp();
                    const uint32_t cnt = __popc(mk);
                    if (row_in)
                        for (uint32_t k = 0; k < cnt; ++k) {
                            const int cx = (int)s_cx[wb + k];
                            if (cx < w.lo[0] || cx > w.hi[0]) continue;
                            const float4 q2 = s_q[wb + k];
                            const float d2 = dist2(q2);
                            if (!(d2 > 0.0f)) {
                                ++zeros;
                                continue;
                            }
                            if (d2 < h_lt2) add(q2, d2, s_mr[wb + k]);
                        }
                    __syncwarp();
                }
            }
        nn = in_window - zeros;
    } else if (active) {
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy) {
                uint32_t beg, end, c;
                row_range(w.lo[0], w.hi[0], yy, zz, beg, end, c);
                for (uint32_t i = beg; i < end; ++i) {
                    const float4 q = __ldg(&sorted[i]);
                    const float d2 = dist2(q);
                    if (!(d2 > 0.0f)) continue;
                    ++nn;
                    if (d2 < h_lt2) add(q, d2, __fdiv_rn(mass, q.w));
                }
            }
    }
    if (!active) return;
    const bool s = nn < 25u || __fsqrt_rn(dot3_rn(sx, sy, sz)) > 3.0f;
    psurf[t] = s ? 1 : 0;
}

// ------------------------------------------------------------ band
// estimationOfSurfaceVertices (cu:554-595): vertices in the clamped box
// idx-3 .. idx+3 (x upper bound exclusive) within 1.5h of a surface
// particle.  `thr` is the largest float whose double value is below
// 1.5*h, so dist <= thr reproduces the reference's double comparison; the
// kernel tests the squared distance against thr2 = sqrt_threshold(thr,
// true), the same decision without the square root.
// Each (y,z) row of at most 6 vertices is OR-ed into the bitset with at most
// two atomics.
__global__ void k_band_stamp(const float4* __restrict__ sorted, const uint32_t* __restrict__ skeys,
                             const uint8_t* __restrict__ surf, const uint8_t* __restrict__ psurf, uint32_t n,
                             Grid sc, float thr2, uint32_t* __restrict__ bits, Counters* ctr)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    bool is_s = false;
    if (t < n) is_s = psurf ? psurf[t] != 0 : surf[skeys[t]] != 0;
    warp_count(&ctr->n_surface, is_s);
    if (!is_s) return;
    const float4 p = sorted[t];
    const Window w = window(cell1(p.x, sc.min[0], sc.cs), cell1(p.y, sc.min[1], sc.cs),
                            cell1(p.z, sc.min[2], sc.cs), 3, sc);
    if (w.hi[0] <= w.lo[0]) return;
    for (int z = w.lo[2]; z <= w.hi[2]; ++z) {
        const float dz = __fsub_rn(vpos1(z, sc.min[2], sc.cs), p.z);
        for (int y = w.lo[1]; y <= w.hi[1]; ++y) {
            const float dy = __fsub_rn(vpos1(y, sc.min[1], sc.cs), p.y);
            const uint32_t v0 = lin3(w.lo[0], y, z, sc);
            const uint32_t word0 = v0 >> 5;
            uint32_t m0 = 0, m1 = 0;
            for (int x = w.lo[0]; x < w.hi[0]; ++x) {
                const float dx = __fsub_rn(vpos1(x, sc.min[0], sc.cs), p.x);
                // sqrt_rn(d2) <= thr  <=>  d2 < thr2 (the smallest float whose root exceeds thr)
                if (dot3_rn(dx, dy, dz) < thr2) {
                    const uint32_t v = v0 + (uint32_t)(x - w.lo[0]);
                    if ((v >> 5) == word0) m0 |= 1u << (v & 31u);
                    else m1 |= 1u << (v & 31u);
                }
            }
            if (m0) atomicOr(bits + word0, m0);
            if (m1) atomicOr(bits + word0 + 1, m1);
        }
    }
}

// compactSurfaceVertex (cu:293-304) over the bitset: every set bit writes
// its vertex id at its rank.  The band vertices also mark their window
// groups (the spatial cell a vertex's FP32 position falls in, as the grouped
// field kernels' group boxes have it); the first mark of a group appends it
// to the group list.  A word is cut into its grid rows; per row the groups
// from the first set bit's to the last's are marked (a superset at worst:
// a marked group without band vertices is found empty).
__global__ void k_band_list(const uint32_t* __restrict__ bits, const uint32_t* __restrict__ prefix,
                            uint32_t nwords, uint32_t* __restrict__ sv, uint32_t cap, GroupMark gm, Counters* ctr)
{
    const uint32_t kx = gm.sp.res[0] + 1, ky = gm.sp.res[1] + 1;
    const uint32_t rx = gm.sc.res[0], rxy = gm.sc.res[0] * gm.sc.res[1];
    const uint32_t nb = ctr->n_band;
    if (blockIdx.x == 0 && threadIdx.x == 0 && nb > cap) {
        atomicOr(&ctr->overflow, 1u);
        atomicMax(&ctr->need_band, nb);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += gridDim.x * blockDim.x) {
        const uint32_t w0 = bits[i];
        if (w0 == 0u) continue;
        uint32_t w = w0;
        uint32_t r = prefix[i];
        while (w) {
            const uint32_t b = __ffs(w) - 1;
            w &= w - 1;
            if (r < cap) sv[r] = (i << 5) | b;
            ++r;
        }
        // the word's rows: bits [s, e) lie in row (y, z) from column x on
        const uint32_t v0 = i << 5;
        uint32_t z = v0 / rxy, y = (v0 - z * rxy) / rx, x = v0 - z * rxy - y * rx;
        uint32_t last = 0xffffffffu;
        for (uint32_t s = 0; s < 32u;) {
            const uint32_t len = min(32u - s, rx - x);
            const uint32_t seg = w0 & ((len == 32u ? 0xffffffffu : ((1u << len) - 1u)) << s);
            if (seg) {
                const uint32_t xf = x + (uint32_t)(__ffs(seg) - 1) - s, xl = x + (31u - (uint32_t)__clz(seg)) - s;
                const int cf = clampi(cell1(vpos1(xf, gm.sc.min[0], gm.sc.cs), gm.sp.min[0], gm.sp.cs), 0, (int)kx - 1);
                const int cl = clampi(cell1(vpos1(xl, gm.sc.min[0], gm.sc.cs), gm.sp.min[0], gm.sp.cs), 0, (int)kx - 1);
                const int cy = clampi(cell1(vpos1(y, gm.sc.min[1], gm.sc.cs), gm.sp.min[1], gm.sp.cs), 0, (int)ky - 1);
                const int cz = clampi(cell1(vpos1(z, gm.sc.min[2], gm.sc.cs), gm.sp.min[2], gm.sp.cs), 0,
                                      (int)gm.sp.res[2]);
                for (int cx = cf; cx <= cl; ++cx) {
                    const uint32_t g = (uint32_t)cx + kx * ((uint32_t)cy + ky * (uint32_t)cz);
                    if (g != last) {
                        last = g;
                        if (atomicExch(gm.gflag + g, 1u) == 0u) gm.glist[atomicAdd(&ctr->n_groups, 1u)] = g;
                    }
                }
            }
            s += len;
            x = 0;
            if (++y == gm.sc.res[1]) {
                y = 0;
                ++z;
            }
        }
    }
}


// Stages the warp's next chunk of candidates [base, end): the ones within
// the box's reach go to sq in their order; returns how many.  nbox is the
// number inside the grown box itself, which the callers count towards their
// chunk sums exactly as before the reach test was added, so that the sums
// join their totals at the same points.
__device__ __forceinline__ uint32_t stage_in_box(const float4* __restrict__ src, uint32_t base, uint32_t end,
                                                 const WarpBox& box, float4* sq, int lane, uint32_t& nbox)
{
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    bool in = false, keep = false;
    if (base + lane < end) {
        q = __ldg(&src[base + lane]);
        in = box.holds(q);
        keep = in && box.reaches(q);
    }
    nbox = __popc(__ballot_sync(0xffffffffu, in));
    const uint32_t m = __ballot_sync(0xffffffffu, keep);
    if (keep) sq[__popc(m & ((1u << lane) - 1u))] = q;
    return __popc(m);
}

// ------------------------------------------------------------ anisotropic path
// calculationOfMeanAndSmoothParticles (cu:598-658).  Two means per particle:
// * mean32: the reference's FP32 sum sum(w x) / sum(w) in its order with its
//   roundings.  It decides the neighbour counts of the covariance stage, so
//   it must be the reference's bit for bit.
// * mean: the same quantity to near FP64 accuracy, as x_i + sum(w (x_j -
//   x_i)) / sum(w).  The offsets x_j - x_i are exact (Sterbenz) and at most R
//   long, so their sums stay small; they are summed per chunk of 32 to 63
//   candidates and the chunk sums, like the weights, are added with Kahan
//   compensation (neighbouring particles sum nearly the same candidates in
//   the same order, so the rounding errors of long plain sums would be
//   correlated between them and would not average out in the field).  The reference's own FP32 sum of absolute coordinates is
//   off by up to 4.5e-7 (1M-particle frame) and by more with thousands of
//   neighbours; the covariance is taken about this mean, and the smoothed
//   positions are formed from it.  mean.w = its weight sum (the adjoint
//   divides by it); smoothed.w = m / rho.
#ifndef FSR_SMOOTH_MIN_BLOCKS
#define FSR_SMOOTH_MIN_BLOCKS 4  // 64 registers: 4 blocks of 256 threads per SM (measured best of 1, 4, 5, 6)
#endif
__global__ void __launch_bounds__(kThreads, FSR_SMOOTH_MIN_BLOCKS) k_smooth(const float4* __restrict__ sorted, uint32_t n,
                                                     const uint2* __restrict__ ranges, Grid sp, float R,
                                                     float R_rcp, float R_lt2, int coop_ok, float one_minus_lambda,
                                                     float lambda, float mass, float4* __restrict__ mean,
                                                     float4* __restrict__ mean32, float4* __restrict__ smoothed)
{
    __shared__ float4 s_q[kThreads];  // 32 staged candidates per warp
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = t < n;
    if (__all_sync(0xffffffffu, !active)) return;
    const int lane = threadIdx.x & 31;
    float4* sq = s_q + (threadIdx.x & ~31u);
    const float4 p = active ? sorted[t] : make_float4(0.f, 0.f, 0.f, 1.f);
    // cells beyond R on some axis only hold zero-weight particles, whose +0
    // terms leave the exact sums unchanged: skip them
    const Window w = narrow(window(cell1(p.x, sp.min[0], sp.cs), cell1(p.y, sp.min[1], sp.cs),
                                   cell1(p.z, sp.min[2], sp.cs), 2, sp),
                            p.x, p.y, p.z, cull_radius(R, sp.cs), sp);
    float ws = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
    // chunk sums of w and w (x_j - x_i), and their compensated totals
    float cw = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    Kahan tw, tx, ty, tz;
    auto add = [&](const float4& q) {
        const float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y), dz = __fsub_rn(p.z, q.z);
        const float d2 = dot3_rn(dx, dy, dz);
        if (!(d2 < R_lt2)) return;  // d >= R: weight 0, and +0 terms leave the sums unchanged
        const float s = div_exact(__fsqrt_rn(d2), R, R_rcp);
        const float wt = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(s, s), s));
        ws = __fadd_rn(ws, wt);
        mx = __fadd_rn(mx, __fmul_rn(q.x, wt));
        my = __fadd_rn(my, __fmul_rn(q.y, wt));
        mz = __fadd_rn(mz, __fmul_rn(q.z, wt));
        cw = __fadd_rn(cw, wt);
        cx = __fmaf_rn(-wt, dx, cx);
        cy = __fmaf_rn(-wt, dy, cy);
        cz = __fmaf_rn(-wt, dz, cz);
    };
    // the chunk sums join the totals once at least 32 candidates (staged or
    // walked) have been added since the last time
    uint32_t since = 0;
    auto fold = [&]() {
        tw.add(cw);
        tx.add(cx);
        ty.add(cy);
        tz.add(cz);
        cw = cx = cy = cz = 0.f;
        since = 0;
    };
    auto row_range = [&](int x0, int x1, int yy, int zz, uint32_t& beg, uint32_t& end) {
        const uint32_t c0 = lin3(x0, yy, zz, sp);
        beg = kEmpty;
        end = 0;
        for (int xx = 0; xx <= x1 - x0; ++xx) {
            const uint2 r = __ldg(&ranges[c0 + xx]);
            if (r.x != kEmpty) {
                beg = min(beg, r.x);
                end = max(end, r.y);
            }
        }
    };
    // A warp whose windows span at most 4 cells per axis walks their union
    // together: each chunk of 32 candidates is loaded once (one per lane)
    // and every lane tests all of them, so no lane idles on a window of its
    // own.  Exact: a candidate outside a lane's window lies beyond the cull
    // radius of its particle on some axis (coop_ok: that radius is below 2
    // cells, so the +-2 cell window never cuts a lane's narrowed window),
    // and the lane's own candidates keep their window order.
    int ulo[3], uhi[3];
    bool compact = coop_ok != 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ulo[a] = (int)__reduce_min_sync(0xffffffffu, active ? (unsigned)w.lo[a] : 0x7fffffffu);
        uhi[a] = (int)__reduce_max_sync(0xffffffffu, active ? (unsigned)(w.hi[a] + 1) : 0u) - 1;
        compact = compact && uhi[a] - ulo[a] <= 3;
    }
    if (compact) {
        // candidates beyond R of every lane's particle are dropped at staging
        // (their weights are 0: the sums are unchanged)
        const WarpBox box = warp_box(active, p.x, p.y, p.z, cull_radius(R, sp.cs));
        for (int zz = ulo[2]; zz <= uhi[2]; ++zz)
            for (int yy = ulo[1]; yy <= uhi[1]; ++yy) {
                uint32_t beg, end;
                row_range(ulo[0], uhi[0], yy, zz, beg, end);
                for (uint32_t base = beg; base < end; base += 32) {
                    uint32_t nbox;
                    const uint32_t cnt = stage_in_box(sorted, base, end, box, sq, lane, nbox);
                    __syncwarp();
                    for (uint32_t k = 0; k < cnt; ++k) add(sq[k]);
                    since += nbox;
                    if (since >= 32) fold();
                    __syncwarp();
                }
            }
    } else {
        if (!active) return;
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy) {
                uint32_t beg, end;
                row_range(w.lo[0], w.hi[0], yy, zz, beg, end);
                for (uint32_t base = beg; base < end; base += 32) {
                    const uint32_t lim = min(end, base + 32u);
                    for (uint32_t i = base; i < lim; ++i) add(__ldg(&sorted[i]));
                    since += lim - base;
                    if (since >= 32) fold();
                }
            }
    }
    if (!active) return;
    fold();
    // ws >= 1: the particle itself has weight 1
    mx = __fdiv_rn(mx, ws);
    my = __fdiv_rn(my, ws);
    mz = __fdiv_rn(mz, ws);
    mean32[t] = make_float4(mx, my, mz, ws);
    const float W = tw.s - tw.c;
    const float ax = p.x + (tx.s - tx.c) / W, ay = p.y + (ty.s - ty.c) / W, az = p.z + (tz.s - tz.c) / W;
    mean[t] = make_float4(ax, ay, az, W);  // w: the weight sum (the adjoint divides by it)
    smoothed[t] = make_float4(__fadd_rn(__fmul_rn(one_minus_lambda, p.x), __fmul_rn(lambda, ax)),
                              __fadd_rn(__fmul_rn(one_minus_lambda, p.y), __fmul_rn(lambda, ay)),
                              __fadd_rn(__fmul_rn(one_minus_lambda, p.z), __fmul_rn(lambda, az)),
                              __fdiv_rn(mass, p.w));
}

// calculationOfTransformMatricesForParticles (cu:689-827) for every
// particle of an involved cell.  The neighbour count (dist <= r about the
// FP32 mean, cu:746) is exact; the covariance is accumulated in chunk sums
// joined with Kahan compensation (CovChunkAccum); the eigen-decomposition
// runs in FP32 and is redone in FP64 when the covariance's condition number
// exceeds 1e4.
// Output record per particle: (x,y,z smoothed, r2max) (G row 0, coef)
// (G row 1, 0) (G row 2, 0) with coef = sigma det(G) m / rho.
// Blocks of two warps: a warp without involved particles exits at once, and
// a small block gives its registers back as soon as its two warps are done,
// so the working warps' blocks fill the SM.
// P lanes per particle: each takes every P-th candidate of the particle's
// walk and the lanes' sums and counts are joined at the end (the covariance
// sums may be taken in any order, the count is an integer).  P = 4 for
// small frames, whose particles alone are too few warps to fill the GPU; P
// = 1 otherwise (four lanes measured slower once the GPU is full).
constexpr int kCovThreads = 64;
constexpr uint32_t kCovSplitBelow = 1u << 17;  // particles below which P = 4
#ifndef FSR_COV_MIN_BLOCKS
#define FSR_COV_MIN_BLOCKS 16
#endif

template <int P>
__global__ void __launch_bounds__(kCovThreads, FSR_COV_MIN_BLOCKS) k_cov(CovArgs a, Counters* ctr)
{
    __shared__ float4 s_q[kCovThreads];  // 32 staged candidates per warp
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) / P;
    const uint32_t sub = threadIdx.x % P;
    bool act = t < a.n && a.invol[a.skeys[t]];
    warp_count(&ctr->n_involved, act && sub == 0);
    if (__all_sync(0xffffffffu, !act)) return;
    const int lane = threadIdx.x & 31;
    float4* sq = s_q + (threadIdx.x & ~31u);
    const float4 p = act ? a.sorted[t] : make_float4(0.f, 0.f, 0.f, 1.f);
    // m: the compensated mean the covariance is taken about; m32: the
    // reference's FP32 mean, which decides the neighbour count (dist <= r,
    // cu:746).  They differ by the FP32 mean's rounding error, dm.
    const float4 m = act ? a.mean[t] : p;
    float dm;
    {
        const float4 m32 = act ? a.mean32[t] : p;
        dm = sqrtf(fmaf(m.x - m32.x, m.x - m32.x, fmaf(m.y - m32.y, m.y - m32.y, (m.z - m32.z) * (m.z - m32.z))));
    }
    const float cr = cull_radius(a.R, a.sp.cs) + 2.0f * dm;
    // a candidate within R of either mean lies within R + dm of m
    const float pre2 = (a.R * 1.0001f + 2.0f * dm) * (a.R * 1.0001f + 2.0f * dm);
    // |q - m|^2 below in2 (above out2) puts q within (beyond) R of m32 with a
    // margin far above the roundings of both squared distances: only
    // candidates in the shell between them take the reference's test
    const float rin = (a.R - dm) * (1.0f - 1e-5f), rout = (a.R + dm) * (1.0f + 1e-5f);
    const float in2 = rin > 0.f ? rin * rin : 0.f, out2 = rout * rout;
    // the window is centred on the particle's cell (cu:710-716); only
    // particles within R of the means count or weigh, so cells beyond R of
    // them on some axis are skipped
    const Window w = narrow(window(cell1(p.x, a.sp.min[0], a.sp.cs), cell1(p.y, a.sp.min[1], a.sp.cs),
                                   cell1(p.z, a.sp.min[2], a.sp.cs), 2, a.sp),
                            m.x, m.y, m.z, cr, a.sp);
    CovChunkAccum acc;
    uint32_t since = 0;  // candidates taken since the chunk sums last joined the totals
    auto fold = [&]() {
        acc.fold();
        since = 0;
    };
    uint32_t nn = 0;
    // d > R: neither counted nor weighed
    auto take = [&](const float4& q) {
        const float vx = __fsub_rn(q.x, m.x), vy = __fsub_rn(q.y, m.y), vz = __fsub_rn(q.z, m.z);
        const float d2 = dot3_rn(vx, vy, vz);
        if (d2 < in2) {
            ++nn;
        } else if (d2 < out2) {  // rare: m32 is loaded again (L1) rather than kept in registers
            const float4 m32 = a.mean32[t];
            if (dot3_rn(__fsub_rn(q.x, m32.x), __fsub_rn(q.y, m32.y), __fsub_rn(q.z, m32.z)) < a.R_le2) ++nn;
        }
        if (d2 < a.R_lt2) acc.add(vx, vy, vz, div_exact(__fsqrt_rn(d2), a.R, a.R_rcp));
    };
    auto near = [&](const float4& q) {
        return dot3_rn(__fsub_rn(q.x, m.x), __fsub_rn(q.y, m.y), __fsub_rn(q.z, m.z)) < pre2;
    };
    auto row_range = [&](int x0, int x1, int yy, int zz, uint32_t& beg, uint32_t& end) {
        const uint32_t c0 = lin3(x0, yy, zz, a.sp);
        beg = kEmpty;
        end = 0;
        for (int xx = 0; xx <= x1 - x0; ++xx) {
            const uint2 r = __ldg(&a.ranges[c0 + xx]);
            if (r.x != kEmpty) {
                beg = min(beg, r.x);
                end = max(end, r.y);
            }
        }
    };
    // Compact warps walk the union of their windows with staged candidates,
    // as in k_smooth.  Exact when the +-2 cell window never cuts a lane's
    // window narrowed about its mean (the mean lies within R of the particle:
    // launch_cov checks R + cull radius < 2 cells), so every candidate the
    // union adds lies beyond R of that lane's mean.
    int ulo[3], uhi[3];
    bool compact = a.coop_ok != 0;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        ulo[ax] = (int)__reduce_min_sync(0xffffffffu, act ? (unsigned)w.lo[ax] : 0x7fffffffu);
        uhi[ax] = (int)__reduce_max_sync(0xffffffffu, act ? (unsigned)(w.hi[ax] + 1) : 0u) - 1;
        compact = compact && uhi[ax] - ulo[ax] <= 3;
    }
    if (compact) {
        // candidates beyond R of every lane's mean are dropped at staging
        const WarpBox box = warp_box(act, m.x, m.y, m.z, cr);
        for (int zz = ulo[2]; zz <= uhi[2]; ++zz)
            for (int yy = ulo[1]; yy <= uhi[1]; ++yy) {
                uint32_t beg, end;
                row_range(ulo[0], uhi[0], yy, zz, beg, end);
                for (uint32_t base = beg; base < end; base += 32) {
                    uint32_t nbox;
                    const uint32_t cnt = stage_in_box(a.sorted, base, end, box, sq, lane, nbox);
                    __syncwarp();
                    if (act) {
                        uint32_t k = sub;
                        for (; k + 3 * P < cnt; k += 4 * P) {
                            const float4 q0 = sq[k], q1 = sq[k + P], q2 = sq[k + 2 * P], q3 = sq[k + 3 * P];
                            const bool n0 = near(q0), n1 = near(q1), n2 = near(q2), n3 = near(q3);
                            if (n0) take(q0);
                            if (n1) take(q1);
                            if (n2) take(q2);
                            if (n3) take(q3);
                        }
                        for (; k < cnt; k += P) take(sq[k]);
                        since += nbox / P;
                        if (since >= 32) fold();
                    }
                    __syncwarp();
                }
            }
    } else if (act && P > 1) {
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy) {
                uint32_t beg, end;
                row_range(w.lo[0], w.hi[0], yy, zz, beg, end);
                for (uint32_t i = beg + sub; i < end; i += P) {
                    const float4 q = __ldg(&a.sorted[i]);
                    if (near(q)) take(q);
                    if (++since >= 32) fold();
                }
            }
    } else if (act) {
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy) {
                uint32_t beg, end;
                row_range(w.lo[0], w.hi[0], yy, zz, beg, end);
                // four candidates per step
                uint32_t i = beg;
                for (; i + 4 <= end; i += 4) {
                    const float4 q0 = __ldg(&a.sorted[i]), q1 = __ldg(&a.sorted[i + 1]);
                    const float4 q2 = __ldg(&a.sorted[i + 2]), q3 = __ldg(&a.sorted[i + 3]);
                    const bool n0 = near(q0), n1 = near(q1), n2 = near(q2), n3 = near(q3);
                    if (n0) take(q0);
                    if (n1) take(q1);
                    if (n2) take(q2);
                    if (n3) take(q3);
                    since += 4;
                    if (since >= 32) fold();
                }
                for (; i < end; ++i) take(__ldg(&a.sorted[i]));
            }
    }
    fold();
    // join the particle's lanes (every lane of the warp takes part)
#pragma unroll
    for (int o = 1; o < P; o <<= 1) {
        auto join = [&](Kahan& k) {
            const float s = __shfl_xor_sync(0xffffffffu, k.s, o), c = __shfl_xor_sync(0xffffffffu, k.c, o);
            k.add(s - c);
        };
        join(acc.tot.wsum);
        join(acc.tot.c11);
        join(acc.tot.c22);
        join(acc.tot.c33);
        join(acc.tot.c12);
        join(acc.tot.c13);
        join(acc.tot.c23);
        nn += __shfl_xor_sync(0xffffffffu, nn, o);
    }
    if (!act || sub != 0) return;
    const CovAccum& sums = acc.tot;
    float G[9];
    const float rmax = covariance_to_G(sums, nn, a.min_neighbors, a.h, a.h2, a.h_inv, G, &ctr->n_fp64);
    if (a.crec) {  // the normalised covariance for the adjoint (the same expressions as covariance_to_G)
        const bool used = nn >= a.min_neighbors;
        const float iw = used ? 1.0f / sums.wsum.s : 0.f;
        a.crec[2ull * t] = make_float4((a.h2 + sums.c11.s) * iw, sums.c12.s * iw, sums.c13.s * iw, (a.h2 + sums.c22.s) * iw);
        a.crec[2ull * t + 1] = make_float4(sums.c23.s * iw, (a.h2 + sums.c33.s) * iw, sums.wsum.s, used ? 1.f : 0.f);
    }
    const float det = G[0] * G[4] * G[8] + G[1] * G[5] * G[6] + G[2] * G[3] * G[7] - G[0] * G[5] * G[7] -
                      G[1] * G[3] * G[8] - G[2] * G[4] * G[6];
    const float4 sm = a.smoothed[t];
    const float r2 = rmax * rmax * 1.0001f;
    // the cell's reach for the field's cell culling: support radius plus the
    // smoothing displacement (the kernel sits at the smoothed position, which
    // may lie outside the cell's box); positive floats order like their bits
    const float dx = sm.x - p.x, dy = sm.y - p.y, dz = sm.z - p.z;
    const float reach = rmax + sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) * 1.0001f;
    atomicMax(reinterpret_cast<int*>(a.cell_rmax) + a.skeys[t], __float_as_int(reach));
    float4* rec = a.grec + 4ull * t;
    rec[0] = make_float4(sm.x, sm.y, sm.z, r2);
    rec[1] = make_float4(G[0], G[1], G[2], a.sigma * det * sm.w);
    rec[2] = make_float4(G[3], G[4], G[5], 0.f);
    rec[3] = make_float4(G[6], G[7], G[8], 0.f);
    // the field's form of the same kernel: q2 = |G d|^2 = d^T (G^T G) d
    const float m00 = G[0] * G[0] + G[3] * G[3] + G[6] * G[6];
    const float m11 = G[1] * G[1] + G[4] * G[4] + G[7] * G[7];
    const float m22 = G[2] * G[2] + G[5] * G[5] + G[8] * G[8];
    const float m01 = G[0] * G[1] + G[3] * G[4] + G[6] * G[7];
    const float m02 = G[0] * G[2] + G[3] * G[5] + G[6] * G[8];
    const float m12 = G[1] * G[2] + G[4] * G[5] + G[7] * G[8];
    float4* q = a.qrec + 3ull * t;
    q[0] = rec[0];
    q[1] = make_float4(m00, 2.0f * m01, 2.0f * m02, rec[1].w);
    q[2] = make_float4(m11, 2.0f * m12, m22, 0.f);
}

// ------------------------------------------------------------ marching cubes
__device__ __forceinline__ float field_at(const McArgs& a, int x, int y, int z)
{
    if (x < 0 || y < 0 || z < 0 || (uint32_t)x >= a.sc.res[0] || (uint32_t)y >= a.sc.res[1] ||
        (uint32_t)z >= a.sc.res[2])
        return 0.f;  // getValue outside the grid (cuh:410-416)
    const uint32_t v = lin3(x, y, z, a.sc);
    if (!band_has(a.band, v)) return a.fill;
    const uint32_t r = band_rank(a.band, v);
    return r < a.cap_band ? __ldg(a.band.phi + r) : a.fill;  // r >= cap only in a frame that is re-run
}

// detectValidSurfaceCubes (cu:328-364): a band vertex as cube origin is
// valid when all 8 corners are band vertices and the case emits triangles.
__global__ void k_mc_classify(McArgs a, const Counters* ctr)
{
    const uint32_t nb = min(ctr->n_band, a.cap_band);
    const uint32_t rx = a.sc.res[0], rxy = a.sc.res[0] * a.sc.res[1];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += gridDim.x * blockDim.x) {
        const uint32_t v = a.sv[t];
        uint32_t x, y, z;
        unlin3(v, a.sc, x, y, z);
        uint32_t info = 0;
        // the cube's corners as 4 rows of two x-neighbours, (dy, dz) in
        // {0,1}^2: one bitset word (two when the pair straddles a word) and
        // one prefix per row give both memberships and both ranks (the x + 1
        // corner of a row in the band follows its x corner: rank + 1)
        if (x < a.sc.res[0] - 1 && y < a.sc.res[1] - 1 && z < a.sc.res[2] - 1) {
            uint32_t vr[4], wd[4];
            bool all = true;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                vr[r] = v + (uint32_t)(r & 1) * rx + (uint32_t)(r >> 1) * rxy;
                const uint32_t w = vr[r] >> 5, b = vr[r] & 31u;
                wd[r] = __ldg(a.band.bits + w);
                const uint32_t next = b < 31u ? (wd[r] >> (b + 1)) : __ldg(a.band.bits + w + 1);
                all = all && ((wd[r] >> b) & 1u) && (next & 1u);
            }
            if (all) {
                uint32_t cs = 0;
                bool in_cap = true;
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const uint32_t b = vr[r] & 31u;
                    const uint32_t r0 = r == 0 ? t : __ldg(a.band.prefix + (vr[r] >> 5)) + __popc(wd[r] & ((1u << b) - 1u));
                    // ranks beyond the capacity only occur in a frame that overflowed and is re-run
                    if (r0 + 1 >= a.cap_band) {
                        in_cap = false;
                        break;
                    }
                    const int dy = r & 1, dz = r >> 1;
                    const int i0 = dy ? (dz ? 2 : 3) : (dz ? 1 : 0);  // corner (0, dy, dz); (1, dy, dz) is i0 + 4
                    if (__ldg(a.band.phi + r0) <= a.iso) cs |= 1u << i0;
                    if (__ldg(a.band.phi + r0 + 1) <= a.iso) cs |= 1u << (i0 + 4);
                }
                if (in_cap) info = (uint32_t)c_mc.nverts[cs] | (cs << 8);
            }
        }
        a.mc[t] = info;
    }
}

// The marching-cubes offsets in one reduce-then-scan over the classify
// words (generateTriangles' vertex offsets and compactValidSurfaceCubes:
// cu:367-380 with the scans of cu:1154-1172).  Per band position t: vofs[t]
// = the vertices of the cubes before t, and a cube with vertices is listed
// at valid[its rank among such cubes] = t.  Within a 4096-position tile both
// counts fit 16 bits (at most 15 x 4096 vertices), so each element is one
// word, vertices low and cubes high, and the block scans add such words;
// the tile totals are kept apart, as full words.
__device__ __forceinline__ uint32_t mc_pair(uint32_t info)
{
    const uint32_t nv = info & 0xFFu;
    return nv | (nv != 0u ? 0x10000u : 0u);
}

__global__ void __launch_bounds__(kScanThreads) k_mc_tile_reduce(McArgs a, const Counters* ctr, uint32_t* tile_sums,
                                                                 uint32_t ntiles_max)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const uint32_t n = min(ctr->n_band, a.cap_band);
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t base = (uint64_t)tile * kScanTile;
        uint32_t s = 0;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint64_t i = base + k * kScanThreads + threadIdx.x;
            if (i < n) s += mc_pair(__ldg(a.mc + i));
        }
        const uint32_t incl = block_inclusive_scan(s, warp_sums);
        if (threadIdx.x == kScanThreads - 1) {
            tile_sums[tile] = incl & 0xFFFFu;
            tile_sums[ntiles_max + tile] = incl >> 16;
        }
        __syncthreads();
    }
}

// One block: exclusive scans of both tile totals in place; the frame's
// vertex and cube counts, and the pool overflow flags.
__global__ void __launch_bounds__(kScanThreads) k_mc_scan_tile_sums(McArgs a, Counters* ctr, uint32_t* tile_sums,
                                                                    uint32_t ntiles_max)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    __shared__ uint32_t last[2];
    const uint32_t n = min(ctr->n_band, a.cap_band);
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    uint32_t carry[2] = {0u, 0u};
    for (uint32_t b = 0; b < ntiles; b += kScanThreads) {
        const uint32_t i = b + threadIdx.x;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            uint32_t* ts = tile_sums + h * ntiles_max;
            const uint32_t x = i < ntiles ? ts[i] : 0u;
            const uint32_t incl = block_inclusive_scan(x, warp_sums);
            if (i < ntiles) ts[i] = carry[h] + incl - x;
            if (threadIdx.x == kScanThreads - 1) last[h] = incl;
            __syncthreads();
            carry[h] += last[h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ctr->n_mesh_verts = carry[0];
        ctr->n_valid = carry[1];
        if (carry[1] > a.cap_valid) {
            atomicOr(&ctr->overflow, 2u);
            atomicMax(&ctr->need_valid, carry[1]);
        }
        if (carry[0] > a.cap_mesh) {
            atomicOr(&ctr->overflow, 4u);
            atomicMax(&ctr->need_mesh, carry[0]);
        }
    }
}

__global__ void __launch_bounds__(kScanThreads) k_mc_tile_scan(McArgs a, const Counters* ctr,
                                                               const uint32_t* tile_prefix, uint32_t ntiles_max)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    __shared__ uint32_t tile_vals[kScanTile];
    const uint32_t n = min(ctr->n_band, a.cap_band);
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t base = (uint64_t)tile * kScanTile;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t j = k * kScanThreads + threadIdx.x;
            const uint64_t i = base + j;
            tile_vals[j] = i < n ? mc_pair(__ldg(a.mc + i)) : 0u;
        }
        __syncthreads();
        // each thread owns kScanItems consecutive positions
        uint32_t local[kScanItems];
        uint32_t s = 0;
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            local[k] = tile_vals[threadIdx.x * kScanItems + k];
            s += local[k];
        }
        const uint32_t incl = block_inclusive_scan(s, warp_sums);
        uint32_t run = incl - s;  // packed exclusive prefix within the tile
        const uint32_t pv = tile_prefix[tile], pq = tile_prefix[ntiles_max + tile];
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint64_t t = base + threadIdx.x * kScanItems + k;
            if (local[k] != 0u && t < n) {
                const uint32_t q = pq + (run >> 16);
                if (q < a.cap_valid) a.valid[q] = (uint32_t)t;
            }
            tile_vals[threadIdx.x * kScanItems + k] = pv + (run & 0xFFFFu);
            run += local[k];
        }
        __syncthreads();
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t j = k * kScanThreads + threadIdx.x;
            const uint64_t i = base + j;
            if (i < n) a.vofs[i] = tile_vals[j];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void normalize_fast(float n[3])
{
    const float inv = rsqrtf(fmaf(n[0], n[0], fmaf(n[1], n[1], n[2] * n[2])));
    n[0] *= inv;
    n[1] *= inv;
    n[2] *= inv;
}

// fVector3::normalize (MathVector.cpp:5-15): scaled only when longer than 1e-7
__device__ __forceinline__ void normalize_guarded(float n[3])
{
    const float len = sqrtf(fmaf(n[0], n[0], fmaf(n[1], n[1], n[2] * n[2])));
    if (len > 1.0e-7f) {
        const float f = 1.0f / len;
        n[0] *= f;
        n[1] *= f;
        n[2] *= f;
    }
}

// generateTriangles (cu:383-463), or with host_mc the host marching cubes
// of Akinci12 (MarchingCubesCPU.cpp:3-72: no normal sign flip, guarded
// normalisation, epsilon test in double).
// The 32 grid positions a cube's corners and central-difference normals
// read: for each corner row (y, z in {0,1}) x = -1..2 (slots 0-15, the
// corners at x = 0, 1), and above/below each corner column y = -1, 2
// (slots 16-23) and z = -1, 2 (slots 24-31).  Each slot outside the cube
// serves one corner's normal, so that normal is written back over its three
// such slots once it is formed.
__device__ __forceinline__ int mc_corner_slot(int cx, int cy, int cz) { return (cz * 2 + cy) * 4 + cx + 1; }
__device__ __forceinline__ int mc_nx_slot(int cx, int cy, int cz) { return (cz * 2 + cy) * 4 + (cx ? 3 : 0); }
__device__ __forceinline__ int mc_ny_slot(int cx, int cy, int cz) { return 16 + (cz * 2 + cx) * 2 + cy; }
__device__ __forceinline__ int mc_nz_slot(int cx, int cy, int cz) { return 24 + (cy * 2 + cx) * 2 + cz; }

__global__ void __launch_bounds__(kThreads) k_mc_generate(McArgs a, const Counters* ctr)
{
    // per thread: the cube's 32 field values, then corner values and normals
    // ([slot][thread]), so that the cut edges can index them without
    // spilling registers
    __shared__ float s_f[32 * kThreads];
    const uint32_t nq = min(ctr->n_valid, a.cap_valid);
    const uint32_t ntot = ctr->n_mesh_verts;
    if (ntot > a.cap_mesh) return;
    const float sgn = a.host_mc ? 1.0f : (a.iso < 0.0f ? -1.0f : 1.0f);
    const int tid = threadIdx.x, lane = tid & 31, wbase = tid & ~31;
    float* f = s_f + tid;
    auto S = [&](int slot) -> float& { return f[slot * kThreads]; };
    // a warp takes 32 consecutive valid cubes: their vertices are one
    // contiguous run of the output, which the warp then writes with
    // consecutive lanes on consecutive vertices (coalesced stores)
    for (uint32_t q0 = blockIdx.x * blockDim.x + (uint32_t)wbase; q0 < nq; q0 += gridDim.x * blockDim.x) {
        const uint32_t q = q0 + (uint32_t)lane;
        uint32_t cs = 0, nv = 0, base = 0;
        int X = 0, Y = 0, Z = 0;
        if (q < nq) {
            const uint32_t t = a.valid[q];
            const uint32_t info = a.mc[t];
            cs = info >> 8;
            nv = info & 0xFFu;
            base = a.vofs[t];
            uint32_t x, y, z;
            unlin3(a.sv[t], a.sc, x, y, z);
            X = (int)x;
            Y = (int)y;
            Z = (int)z;
            // the 32 positions, each looked up once (the corner-by-corner form
            // reads 56)
            for (int r = 0; r < 4; ++r) {
                const int cy = r & 1, cz = r >> 1;
                for (int xi = 0; xi < 4; ++xi) S(r * 4 + xi) = field_at(a, X + xi - 1, Y + cy, Z + cz);
            }
            for (int k = 0; k < 4; ++k) {
                const int c0 = k & 1, c1 = k >> 1;
                S(16 + k * 2) = field_at(a, X + c0, Y - 1, Z + c1);      // (cx, cz) = (c0, c1)
                S(16 + k * 2 + 1) = field_at(a, X + c0, Y + 2, Z + c1);
                S(24 + k * 2) = field_at(a, X + c0, Y + c1, Z - 1);      // (cx, cy) = (c0, c1)
                S(24 + k * 2 + 1) = field_at(a, X + c0, Y + c1, Z + 2);
            }
            // corner normals, f(p - e) - f(p + e) per axis, over their slots
            for (int i = 0; i < 8; ++i) {
                const int cx = mc::cornerDx(i), cy = mc::cornerDy(i), cz = mc::cornerDz(i);
                float cn[3] = {cx ? S(mc_corner_slot(0, cy, cz)) - S(mc_nx_slot(1, cy, cz))
                                  : S(mc_nx_slot(0, cy, cz)) - S(mc_corner_slot(1, cy, cz)),
                               cy ? S(mc_corner_slot(cx, 0, cz)) - S(mc_ny_slot(cx, 1, cz))
                                  : S(mc_ny_slot(cx, 0, cz)) - S(mc_corner_slot(cx, 1, cz)),
                               cz ? S(mc_corner_slot(cx, cy, 0)) - S(mc_nz_slot(cx, cy, 1))
                                  : S(mc_nz_slot(cx, cy, 0)) - S(mc_corner_slot(cx, cy, 1))};
                if (a.host_mc) normalize_guarded(cn);
                else normalize_fast(cn);
                S(mc_nx_slot(cx, cy, cz)) = cn[0];
                S(mc_ny_slot(cx, cy, cz)) = cn[1];
                S(mc_nz_slot(cx, cy, cz)) = cn[2];
            }
        }
        // the warp's run: the exclusive prefix of its cubes' vertex counts
        uint32_t ex = nv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, ex, o);
            if (lane >= o) ex += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, ex, 31);
        ex -= nv;
        const uint32_t run0 = __shfl_sync(0xffffffffu, base, 0);  // lane 0 holds a cube (q0 < nq)
        __syncwarp();
        for (uint32_t jb = 0; jb < total; jb += 32) {
            const uint32_t j = jb + (uint32_t)lane;
            // the cube of vertex j: the last lane whose run starts at or before j
            int c = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const uint32_t e = __shfl_sync(0xffffffffu, ex, (c + step) & 31);
                if (c + step < 32 && e <= j) c += step;
            }
            const uint32_t k = j - __shfl_sync(0xffffffffu, ex, c);
            const uint32_t ccs = __shfl_sync(0xffffffffu, cs, c);
            const int cX = __shfl_sync(0xffffffffu, X, c), cY = __shfl_sync(0xffffffffu, Y, c),
                      cZ = __shfl_sync(0xffffffffu, Z, c);
            if (j >= total) continue;
            const float* g = s_f + wbase + c;  // that cube's slots
            auto G = [&](int slot) { return g[slot * kThreads]; };
            const int e = (int)((c_mc.tri[ccs] >> (4u * k)) & 0xFu);
            const int i0 = mc::edgeA(e), i1 = mc::edgeB(e);
            const int a0x = mc::cornerDx(i0), a0y = mc::cornerDy(i0), a0z = mc::cornerDz(i0);
            const int a1x = mc::cornerDx(i1), a1y = mc::cornerDy(i1), a1z = mc::cornerDz(i1);
            const float v0 = G(mc_corner_slot(a0x, a0y, a0z)), v1 = G(mc_corner_slot(a1x, a1y, a1z));
            const float d = v1 - v0;
            const float fr = (d > -1.0e-7f && d < 1.0e-7f) ? 0.5f : (a.iso - v0) / d;
            const int c0[3] = {cX + a0x, cY + a0y, cZ + a0z};
            const int c1[3] = {cX + a1x, cY + a1y, cZ + a1z};
            float ip[3], in[3];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                const float p0 = vpos1(c0[kk], a.sc.min[kk], a.sc.cs), p1 = vpos1(c1[kk], a.sc.min[kk], a.sc.cs);
                ip[kk] = fmaf(fr, p1 - p0, p0);
                const float n0 = G(kk == 0 ? mc_nx_slot(a0x, a0y, a0z) : kk == 1 ? mc_ny_slot(a0x, a0y, a0z)
                                                                       : mc_nz_slot(a0x, a0y, a0z));
                const float n1 = G(kk == 0 ? mc_nx_slot(a1x, a1y, a1z) : kk == 1 ? mc_ny_slot(a1x, a1y, a1z)
                                                                       : mc_nz_slot(a1x, a1y, a1z));
                in[kk] = fmaf(fr, n1 - n0, n0);
            }
            if (a.host_mc) normalize_guarded(in);
            else normalize_fast(in);
            const uint64_t o = 3ull * (run0 + j);
            a.out_pos[o] = ip[0];
            a.out_pos[o + 1] = ip[1];
            a.out_pos[o + 2] = ip[2];
            a.out_nrm[o] = sgn * in[0];
            a.out_nrm[o + 1] = sgn * in[1];
            a.out_nrm[o + 2] = sgn * in[2];
            if (a.out_key) {
                // the edge's lower end point and its axis (the one coordinate
                // in which the two corners differ)
                const uint32_t lx = (uint32_t)min(c0[0], c1[0]), ly = (uint32_t)min(c0[1], c1[1]),
                               lz = (uint32_t)min(c0[2], c1[2]);
                const uint32_t axis = c0[0] != c1[0] ? 0u : (c0[1] != c1[1] ? 1u : 2u);
                const uint64_t lin = (uint64_t)lx + (uint64_t)a.sc.res[0] * ((uint64_t)ly + (uint64_t)a.sc.res[1] * lz);
                a.out_key[run0 + j] = 3ull * lin + axis;
            }
        }
        __syncwarp();  // the next cubes overwrite the slots
    }
}

__global__ void k_particle_flags(const uint32_t* __restrict__ skeys, const uint8_t* __restrict__ surf,
                                 const uint8_t* __restrict__ psurf, uint32_t n, uint32_t* __restrict__ out)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    out[t] = psurf ? psurf[t] : surf[skeys[t]];
}

}  // namespace

// ------------------------------------------------------------ launchers

// Smallest float x >= 0 whose correctly rounded square root is >= R
// (strict = false) or > R (strict = true): for d2 >= 0,
//   sqrt_rn(d2) <  R  <=>  d2 < threshold(R, false)
//   sqrt_rn(d2) <= R  <=>  d2 < threshold(R, true)
// so the kernels test distances without a square root and take the root
// only where the weight needs it.  sqrtf on the host and __fsqrt_rn on the
// device are both the IEEE correctly rounded square root.
float sqrt_threshold(float R, bool strict)
{
    auto ok = [&](float x) { return strict ? std::sqrt(x) > R : std::sqrt(x) >= R; };
    float x = R * R;
    if (!(x > 0.0f) || !std::isfinite(x)) return x;
    while (x > 0.0f && ok(std::nextafterf(x, 0.0f))) x = std::nextafterf(x, 0.0f);
    while (!ok(x)) x = std::nextafterf(x, INFINITY);
    return x;
}

void launch_hash(const KernelCtx& c, const float* xyz, uint32_t n, const Grid& sp, uint32_t* keys,
                 uint32_t* vals, Counters* ctr)
{
    if (!n) return;
    k_hash<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(xyz, n, sp, keys, vals, ctr);
    ++g_launches;
}

void launch_ranges_gather(const KernelCtx& c, const uint32_t* skeys, const uint32_t* perm, uint32_t n,
                          const float* xyz, const float* dens, float4* sorted, uint2* ranges, uint8_t* occ)
{
    if (!n) return;
    k_ranges_gather<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(skeys, perm, n, xyz, dens, sorted, ranges, occ);
    ++g_launches;
}

void launch_density(const KernelCtx& c, float4* sorted, uint32_t n, const uint2* ranges, const Grid& sp, float h,
                    float mass, float* rho)
{
    if (n == 0) return;
    const int ext = std::max(1, (int)std::ceil((double)h * 1.0001 / sp.cs + 1e-4));
    const float h2 = h * h;
    const float sigma = 315.0f / (64.0f * 3.1415926535898f);
    const float scale = mass * sigma / (h * h * h);
    k_density<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(sorted, n, ranges, sp, ext, h, h2, 1.0f / h2, scale, rho);
    k_set_density<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(sorted, rho, n);
    g_launches += 2;
}

void launch_surface_cells(const KernelCtx& c, const Grid& sp, const uint8_t* occ, uint8_t* surf)
{
    const uint64_t C = (uint64_t)sp.res[0] * sp.res[1] * sp.res[2];
    k_surface_cells<<<blocks_for(C, bs(c)), bs(c), 0, c.stream>>>(sp, occ, surf);
    ++g_launches;
}

void launch_involved_cells(const KernelCtx& c, const Grid& sp, const uint8_t* occ, const uint8_t* surf,
                           uint8_t* invol)
{
    const uint64_t C = (uint64_t)sp.res[0] * sp.res[1] * sp.res[2];
    k_involved_cells<<<blocks_for(C, bs(c)), bs(c), 0, c.stream>>>(sp, occ, surf, invol);
    ++g_launches;
}

void launch_colorfield(const KernelCtx& c, const float4* sorted, uint32_t n, const uint2* ranges,
                       const uint32_t* skeys, const Grid& sp, float h, float h2, float mass, uint8_t* psurf)
{
    if (!n) return;
    // -45 / (pi h^4) exactly as the reference evaluates it in double
    const double k = -45.0 / (3.1415926535 * (double)h2 * (double)h2);
    // the FP32 form of the gradient needs |k| x^2 (x in (0, 1]) to stay a
    // normal float: |k| within [1e-20, 1e30]; else the double expression
    const double K = -k;
    float khi = 0.f, klo = 0.f;
    if (K >= 1e-20 && K <= 1e30) {
        khi = (float)K;
        klo = (float)(K - (double)khi);
    }
    k_colorfield<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(sorted, n, ranges, skeys, sp, h, 1.0f / h,
                                                           sqrt_threshold(h, false), k, khi, klo, mass, psurf);
    ++g_launches;
}

void launch_band_stamp(const KernelCtx& c, const float4* sorted, const uint32_t* skeys, const uint8_t* surf,
                       const uint8_t* psurf, uint32_t n, const Grid& sc, float thr, uint32_t* bits,
                       Counters* ctr)
{
    if (!n) return;
    k_band_stamp<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(sorted, skeys, surf, psurf, n, sc,
                                                           sqrt_threshold(thr, true), bits, ctr);
    ++g_launches;
}

void launch_band_list(const KernelCtx& c, const uint32_t* bits, const uint32_t* prefix, uint32_t nwords,
                      uint32_t* sv, uint32_t cap, const GroupMark& gm, Counters* ctr)
{
    k_band_list<<<persistent_blocks(c, nwords, 16), bs(c), 0, c.stream>>>(bits, prefix, nwords, sv, cap, gm, ctr);
    ++g_launches;
}


void launch_smooth(const KernelCtx& c, const float4* sorted, uint32_t n, const uint2* ranges, const Grid& sp,
                   float R, float lambda, float mass, float4* mean, float4* mean32, float4* smoothed)
{
    if (!n) return;
    // (1.0 - lambda) is evaluated in double and rounded (cu:656)
    const float oml = (float)(1.0 - (double)lambda);
    // warps may walk the union of their windows when the cull radius stays
    // below two cells (see k_smooth)
    const int coop_ok = (R * 1.0001f + 1e-4f * sp.cs) < 2.0f * sp.cs * 0.9999f ? 1 : 0;
    k_smooth<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(sorted, n, ranges, sp, R, 1.0f / R, sqrt_threshold(R, false),
                                                       coop_ok, oml, lambda, mass, mean, mean32,
                                                       smoothed);
    ++g_launches;
}

void launch_cov(const KernelCtx& c, const CovArgs& a0, Counters* ctr)
{
    if (!a0.n) return;
    CovArgs a = a0;
    a.R_lt2 = sqrt_threshold(a.R, false);
    a.R_rcp = 1.0f / a.R;
    a.R_le2 = sqrt_threshold(a.R, true);
    a.coop_ok = (a.R + a.R * 1.0001f + 1e-4f * a.sp.cs) < 2.0f * a.sp.cs * 0.9999f ? 1 : 0;
    if (a.n < kCovSplitBelow)
        k_cov<4><<<blocks_for((uint64_t)a.n * 4, kCovThreads), kCovThreads, 0, c.stream>>>(a, ctr);
    else
        k_cov<1><<<blocks_for(a.n, kCovThreads), kCovThreads, 0, c.stream>>>(a, ctr);
    ++g_launches;
}

void launch_mc_classify(const KernelCtx& c, const McArgs& a, Counters* ctr)
{
    k_mc_classify<<<persistent_blocks(c, a.cap_band, 16), bs(c), 0, c.stream>>>(a, ctr);
    ++g_launches;
}

size_t mc_offsets_scratch_words(uint32_t cap_band)
{
    return 2 * (size_t)((cap_band + kScanTile - 1) / kScanTile) + 2;
}

void launch_mc_offsets(const KernelCtx& c, const McArgs& a, Counters* ctr, uint32_t* scratch)
{
    const uint32_t ntiles_max = (a.cap_band + kScanTile - 1) / kScanTile;
    const uint32_t g = std::max<uint32_t>(1, std::min<uint32_t>(ntiles_max, 65535));
    k_mc_tile_reduce<<<g, kScanThreads, 0, c.stream>>>(a, ctr, scratch, ntiles_max);
    k_mc_scan_tile_sums<<<1, kScanThreads, 0, c.stream>>>(a, ctr, scratch, ntiles_max);
    k_mc_tile_scan<<<g, kScanThreads, 0, c.stream>>>(a, ctr, scratch, ntiles_max);
    g_launches += 3;
}

void launch_mc_generate(const KernelCtx& c, const McArgs& a, Counters* ctr)
{
    k_mc_generate<<<persistent_blocks(c, a.cap_valid, 16), bs(c), 0, c.stream>>>(a, ctr);
    ++g_launches;
}

void launch_particle_flags(const KernelCtx& c, const uint32_t* skeys, const uint8_t* surf, const uint8_t* psurf,
                           uint32_t n, uint32_t* out)
{
    if (!n) return;
    k_particle_flags<<<blocks_for(n, bs(c)), bs(c), 0, c.stream>>>(skeys, surf, psurf, n, out);
    ++g_launches;
}

}  // namespace fsr
