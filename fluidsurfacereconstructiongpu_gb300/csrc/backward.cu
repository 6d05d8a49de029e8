// Adjoint (backward) kernels: gradient of a scalar loss through the last
// frame's triangle soup back to the particle positions, with the discrete
// structure of the frame held fixed (sorted order, band, valid cubes and MC
// cases, neighbourhoods, isolated-particle decisions, FP64 re-solves).
//
//   mesh vertex p = p_a + f (p_b - p_a), f = (iso - phi_a) / (phi_b - phi_a)
//     -> dL/dphi at the two corners of each edge (k_mc_backward)
//   ZB05:  phi = |xbar - v| - r_p, xbar = sum w x / sum w, w = (1 - d^2/h^2)^3
//   TC01:  phi = sum t^2 - t + 1/4, t = d^2 / 2h^2
//   Yu13:  phi = sum c_j (1 - |G_j (x~_j - v)|^2)^3 - 1/2, c_j = sigma det(G_j) m/rho_j
//          (unscaled kernel with G = I, c = sigma m/rho for non-involved particles)
//     -> dL/dx (ZB05, TC01) or dL/dx~ and dL/dG (Yu13), gathered per particle
//        over the band vertices of its support and window (k_field_backward_*)
//   G = (1/h) cbrt(s1 s2 s3) V diag(1/s) V^T, s = eigenvalues of C clamped
//       from below at max/4, C = (h^2 I + sum w v v^T) / sum w, v = x_j - mean
//     -> dL/dC by the derivative of a spectral function (Daleckii-Krein form
//        with the cross terms of the clamp and of the volume factor), then
//        dL/dx_j and dL/dmean over the neighbours, recomputed (k_cov_backward)
//   x~ = (1 - lambda) x + lambda mean, mean = sum w x / sum w, w = 1 - (d/R)^3
//     -> dL/dx over the neighbours, recomputed (k_smooth_backward)
// Neighbour gradients are added with atomics (their order is not fixed; the
// results agree with finite differences within FP32 rounding).
#include "backward.h"

#include "cov_solver.cuh"

#include <algorithm>

namespace fsr {
namespace {

constexpr int kT = 256;

// ---------------------------------------------------------------- MC
__global__ void k_mc_backward(BwdArgs a, const Counters* ctr)
{
    const uint32_t nq = min(ctr->n_valid, a.cap_valid);
    const uint32_t rx = a.sc.res[0], rxy = a.sc.res[0] * a.sc.res[1];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const uint32_t t = a.valid[q];
        const uint32_t info = a.mc[t];
        const uint32_t cs = info >> 8, nv = info & 0xFFu, base = a.vofs[t];
        const uint32_t v = a.sv[t];
        uint32_t rk[8];
        float val[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const uint32_t id = v + (uint32_t)mc::cornerDx(i) + (uint32_t)mc::cornerDy(i) * rx +
                                (uint32_t)mc::cornerDz(i) * rxy;
            rk[i] = band_rank(a.band, id);
            val[i] = __ldg(a.band.phi + rk[i]);
        }
        const uint64_t tri = a.tri[cs];
        for (uint32_t k = 0; k < nv; ++k) {
            const int e = (int)((tri >> (4u * k)) & 0xFu);
            const int ia = mc::edgeA(e), ib = mc::edgeB(e);
            float fa = 0.f, fb = 0.f;
            uint32_t ra = 0, rb = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (i == ia) { fa = val[i]; ra = rk[i]; }
                if (i == ib) { fb = val[i]; rb = rk[i]; }
            }
            const float d = fb - fa;
            if (d > -1.0e-7f && d < 1.0e-7f) continue;  // f = 0.5 is constant there
            // p_b - p_a is one grid spacing along the edge's axis
            const int ax = mc::cornerDx(ib) != mc::cornerDx(ia) ? 0 : (mc::cornerDy(ib) != mc::cornerDy(ia) ? 1 : 2);
            const int sgn = (ax == 0 ? mc::cornerDx(ib) - mc::cornerDx(ia)
                                     : ax == 1 ? mc::cornerDy(ib) - mc::cornerDy(ia) : mc::cornerDz(ib) - mc::cornerDz(ia));
            const float gp = a.gmesh[3ull * (base + k) + ax];
            const float gf = gp * (float)sgn * a.sc.cs;
            const float inv = 1.0f / (d * d);
            atomicAdd(a.gphi + ra, gf * (a.iso - fb) * inv);
            atomicAdd(a.gphi + rb, -gf * (a.iso - fa) * inv);
        }
    }
}

// keys (window centres) holding a band vertex with a non-zero field gradient;
// the first vertex to mark a key appends it to the list the grouped
// adjoints take their groups from
__global__ void k_mark_keys(BwdArgs a, const Counters* ctr)
{
    const uint32_t nb = min(ctr->n_band, a.cap_band);
    const uint32_t kx = a.sp.res[0] + 1, ky = a.sp.res[1] + 1;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += gridDim.x * blockDim.x) {
        if (a.gphi[t] == 0.f) continue;
        uint32_t x, y, z;
        unlin3(a.sv[t], a.sc, x, y, z);
        const int cx = cell1(vpos1(x, a.sc.min[0], a.sc.cs), a.sp.min[0], a.sp.cs);
        const int cy = cell1(vpos1(y, a.sc.min[1], a.sc.cs), a.sp.min[1], a.sp.cs);
        const int cz = cell1(vpos1(z, a.sc.min[2], a.sc.cs), a.sp.min[2], a.sp.cs);
        const uint32_t key = ((uint32_t)cz * ky + cy) * kx + cx;
        if (a.gkey[key] == 0u && atomicExch(&a.gkey[key], 1u) == 0u) a.glist[4 + atomicAdd(&a.glist[0], 1u)] = key;
    }
}

// Does any key within +-ext of the particle's cell hold a gradient vertex?
__device__ __forceinline__ bool near_gradient(const BwdArgs& a, int cx, int cy, int cz, int ext)
{
    const int kx = (int)a.sp.res[0] + 1, ky = (int)a.sp.res[1] + 1, kz = (int)a.sp.res[2] + 1;
    for (int z = max(cz - ext, 0); z <= min(cz + ext, kz - 1); ++z)
        for (int y = max(cy - ext, 0); y <= min(cy + ext, ky - 1); ++y)
            for (int x = max(cx - ext, 0); x <= min(cx + ext, kx - 1); ++x)
                if (a.gkey[((uint32_t)z * ky + y) * kx + x]) return true;
    return false;
}

// Visits every band vertex with a non-zero field gradient inside the vertex
// index box [lo, hi] (inclusive): fn(rank, gphi, vx, vy, vz).
template <class Fn>
__device__ __forceinline__ void for_band_vertices(const BwdArgs& a, const int lo[3], const int hi[3], Fn fn)
{
    const int n = hi[0] - lo[0] + 1;
    if (n <= 0 || hi[1] < lo[1] || hi[2] < lo[2]) return;
    for (int z = lo[2]; z <= hi[2]; ++z) {
        const float vz = vpos1(z, a.sc.min[2], a.sc.cs);
        for (int y = lo[1]; y <= hi[1]; ++y) {
            const float vy = vpos1(y, a.sc.min[1], a.sc.cs);
            const uint32_t v0 = lin3(lo[0], y, z, a.sc);
            const uint32_t v1 = v0 + (uint32_t)n;  // exclusive
            for (uint32_t w = v0 >> 5; w <= (v1 - 1) >> 5; ++w) {
                uint32_t bits = __ldg(a.band.bits + w);
                const uint32_t wbase = w << 5;
                if (wbase < v0) bits &= ~0u << (v0 - wbase);
                if (v1 - wbase < 32u) bits &= (1u << (v1 - wbase)) - 1u;
                if (!bits) continue;
                const uint32_t pre = __ldg(a.band.prefix + w);
                const uint32_t word = __ldg(a.band.bits + w);
                while (bits) {
                    const uint32_t b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const uint32_t rank = pre + __popc(word & ((1u << b) - 1u));
                    if (rank >= a.cap_band) continue;
                    const float g = a.gphi[rank];
                    if (g == 0.f) continue;
                    const int x = lo[0] + (int)(wbase + b - v0);
                    fn(rank, g, vpos1(x, a.sc.min[0], a.sc.cs), vy, vz);
                }
            }
        }
    }
}

// Vertex index box of the particle's reverse window (vertices whose window,
// centred on their FP32 cell, contains cell c) intersected with the box of
// grid vertices within r of point p.
__device__ __forceinline__ void window_box(const BwdArgs& a, const int c[3], int ext, const float p[3], float r,
                                           int lo[3], int hi[3])
{
    const int w0[3] = {first_vertex<0>(max(c[0] - ext, 0), a.sc, a.sp, a.ratio),
                       first_vertex<1>(max(c[1] - ext, 0), a.sc, a.sp, a.ratio),
                       first_vertex<2>(max(c[2] - ext, 0), a.sc, a.sp, a.ratio)};
    const int w1[3] = {first_vertex<0>(c[0] + ext + 1, a.sc, a.sp, a.ratio) - 1,
                       first_vertex<1>(c[1] + ext + 1, a.sc, a.sp, a.ratio) - 1,
                       first_vertex<2>(c[2] + ext + 1, a.sc, a.sp, a.ratio) - 1};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float inv = 1.0f / a.sc.cs;
        const int s0 = __float2int_rd((p[k] - r - a.sc.min[k]) * inv);
        const int s1 = __float2int_ru((p[k] + r - a.sc.min[k]) * inv);
        lo[k] = max(w0[k], s0);
        hi[k] = min(w1[k], s1);
    }
}

// ---------------------------------------------------------------- ZB05 / TC01 field
template <bool TC01>
__global__ void k_field_backward_iso(BwdArgs a)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    const float4 q = a.sorted[j];
    const int c[3] = {cell1(q.x, a.sp.min[0], a.sp.cs), cell1(q.y, a.sp.min[1], a.sp.cs),
                      cell1(q.z, a.sp.min[2], a.sp.cs)};
    float gx = 0.f, gy = 0.f, gz = 0.f;
    if (near_gradient(a, c[0], c[1], c[2], 1)) {
        const float p[3] = {q.x, q.y, q.z};
        int lo[3], hi[3];
        window_box(a, c, 1, p, cull_radius(a.h, a.sp.cs), lo, hi);
        const float h2 = a.h * a.h, inv_h2 = 1.0f / h2;
        for_band_vertices(a, lo, hi, [&](uint32_t rank, float g, float vx, float vy, float vz) {
            const float dx = q.x - vx, dy = q.y - vy, dz = q.z - vz;
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (TC01) {
                if (d2 > h2) return;
                const float tt = d2 * inv_h2 * 0.5f;
                const float s = g * (2.f * tt - 1.f) * inv_h2;
                gx = fmaf(s, dx, gx);
                gy = fmaf(s, dy, gy);
                gz = fmaf(s, dz, gz);
            } else {
                if (d2 >= h2) return;
                const float4 m = a.mv[rank];  // mean - v, weight sum
                if (!(m.w > 0.f)) return;
                const float ml = sqrtf(fmaf(m.x, m.x, fmaf(m.y, m.y, m.z * m.z)));
                if (!(ml > 0.f)) return;
                const float u = 1.0f - d2 * inv_h2;
                const float wt = u * u * u;
                // d phi / d xbar = (xbar - v) / |xbar - v|
                const float ex = g * m.x / ml, ey = g * m.y / ml, ez = g * m.z / ml;
                // d xbar / d x_j = (w I + (x_j - xbar) (dw/dx_j)^T) / W, dw/dx_j = -6 u^2 (x_j - v) / h^2
                const float proj = ex * (dx - m.x) + ey * (dy - m.y) + ez * (dz - m.z);
                const float k2 = proj * (-6.0f * u * u * inv_h2);
                const float iw = 1.0f / m.w;
                gx += (wt * ex + k2 * dx) * iw;
                gy += (wt * ey + k2 * dy) * iw;
                gz += (wt * ez + k2 * dz) * iw;
            }
        });
    }
    a.gx[j] = make_float4(gx, gy, gz, 0.f);
}

// dL/d(particle radius) of ZB05: -sum of dL/dphi over vertices with weight
__global__ void k_radius_grad(BwdArgs a, const Counters* ctr, float* out)
{
    const uint32_t nb = min(ctr->n_band, a.cap_band);
    float s = 0.f;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += gridDim.x * blockDim.x)
        if (a.mv[t].w > 0.f) s -= a.gphi[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s != 0.f) atomicAdd(out, s);
}

// ---------------------------------------------------------------- anisotropic field
__global__ void k_field_backward_aniso(BwdArgs a)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    const float4 q = a.sorted[j];
    const int c[3] = {cell1(q.x, a.sp.min[0], a.sp.cs), cell1(q.y, a.sp.min[1], a.sp.cs),
                      cell1(q.z, a.sp.min[2], a.sp.cs)};
    const bool involved = a.invol[a.skeys[j]] != 0;
    float gxs = 0.f, gys = 0.f, gzs = 0.f;                    // dL/dx~
    float gg[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // dL/dG without the det term
    float sc = 0.f;                                          // sum of dL/dphi (1 - q2)^3
    if (near_gradient(a, c[0], c[1], c[2], 2)) {
        float4 r0, g0, g1, g2;
        if (involved) {
            r0 = a.grec[4ull * j];
            g0 = a.grec[4ull * j + 1];
            g1 = a.grec[4ull * j + 2];
            g2 = a.grec[4ull * j + 3];
        } else {
            const float4 s = a.smoothed[j];
            r0 = make_float4(s.x, s.y, s.z, 1.0f);
            g0 = make_float4(1.f, 0.f, 0.f, a.sigma * s.w);
            g1 = make_float4(0.f, 1.f, 0.f, 0.f);
            g2 = make_float4(0.f, 0.f, 1.f, 0.f);
        }
        const float coef = g0.w;
        const float p[3] = {r0.x, r0.y, r0.z};
        int lo[3], hi[3];
        window_box(a, c, 2, p, sqrtf(r0.w), lo, hi);
        for_band_vertices(a, lo, hi, [&](uint32_t rank, float g, float vx, float vy, float vz) {
            const float rx = r0.x - vx, ry = r0.y - vy, rz = r0.z - vz;
            const float tx = fmaf(g0.x, rx, fmaf(g0.y, ry, g0.z * rz));
            const float ty = fmaf(g1.x, rx, fmaf(g1.y, ry, g1.z * rz));
            const float tz = fmaf(g2.x, rx, fmaf(g2.y, ry, g2.z * rz));
            const float q2 = fmaf(tx, tx, fmaf(ty, ty, tz * tz));
            if (!(q2 < 1.0f)) return;
            const float u = 1.0f - q2;
            const float A = -6.0f * g * coef * u * u;
            // d/dr of (1 - |G r|^2)^3 = -6 (1 - q2)^2 G^T G r
            gxs += A * (g0.x * tx + g1.x * ty + g2.x * tz);
            gys += A * (g0.y * tx + g1.y * ty + g2.y * tz);
            gzs += A * (g0.z * tx + g1.z * ty + g2.z * tz);
            gg[0] += A * tx * rx; gg[1] += A * tx * ry; gg[2] += A * tx * rz;
            gg[3] += A * ty * rx; gg[4] += A * ty * ry; gg[5] += A * ty * rz;
            gg[6] += A * tz * rx; gg[7] += A * tz * ry; gg[8] += A * tz * rz;
            sc += g * u * u * u;
        });
        if (involved) {
            // c = sigma det(G) m / rho: d c / d G = c G^-T (G is symmetric)
            const float G[9] = {g0.x, g0.y, g0.z, g1.x, g1.y, g1.z, g2.x, g2.y, g2.z};
            const float det = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                              G[2] * (G[3] * G[7] - G[4] * G[6]);
            if (det != 0.f) {
                const float k = sc * coef / det;
                gg[0] += k * (G[4] * G[8] - G[5] * G[7]);
                gg[1] += k * (G[5] * G[6] - G[3] * G[8]);
                gg[2] += k * (G[3] * G[7] - G[4] * G[6]);
                gg[3] += k * (G[2] * G[7] - G[1] * G[8]);
                gg[4] += k * (G[0] * G[8] - G[2] * G[6]);
                gg[5] += k * (G[1] * G[6] - G[0] * G[7]);
                gg[6] += k * (G[1] * G[5] - G[2] * G[4]);
                gg[7] += k * (G[2] * G[3] - G[0] * G[5]);
                gg[8] += k * (G[0] * G[4] - G[1] * G[3]);
            }
        }
    }
    a.gsmooth[j] = make_float4(gxs, gys, gzs, 0.f);
    a.gG[3ull * j] = make_float4(gg[0], gg[1], gg[2], 0.f);
    a.gG[3ull * j + 1] = make_float4(gg[3], gg[4], gg[5], 0.f);
    a.gG[3ull * j + 2] = make_float4(gg[6], gg[7], gg[8], 0.f);
}

// c = sigma det(G) m / rho: adds (sum dL/dphi (1 - q2)^3) dc/dG = that sum
// times c G^-T (G is symmetric) to dL/dG of each involved particle, after
// the grouped adjoint has accumulated the sum in gsmooth.w.
__global__ void k_det_term(BwdArgs a)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n || !a.invol[a.skeys[j]]) return;
    const float sc = a.gsmooth[j].w;
    if (sc == 0.f) return;
    const float4 g0 = a.grec[4ull * j + 1], g1 = a.grec[4ull * j + 2], g2 = a.grec[4ull * j + 3];
    const float G[9] = {g0.x, g0.y, g0.z, g1.x, g1.y, g1.z, g2.x, g2.y, g2.z};
    const float det = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                      G[2] * (G[3] * G[7] - G[4] * G[6]);
    if (det == 0.f) return;
    const float k = sc * g0.w / det;
    float4* r = a.gG + 3ull * j;
    float4 r0 = r[0], r1 = r[1], r2 = r[2];
    r0.x += k * (G[4] * G[8] - G[5] * G[7]);
    r0.y += k * (G[5] * G[6] - G[3] * G[8]);
    r0.z += k * (G[3] * G[7] - G[4] * G[6]);
    r1.x += k * (G[2] * G[7] - G[1] * G[8]);
    r1.y += k * (G[0] * G[8] - G[2] * G[6]);
    r1.z += k * (G[1] * G[6] - G[0] * G[7]);
    r2.x += k * (G[1] * G[5] - G[2] * G[4]);
    r2.y += k * (G[2] * G[3] - G[0] * G[5]);
    r2.z += k * (G[0] * G[4] - G[1] * G[3]);
    r[0] = r0;
    r[1] = r1;
    r[2] = r2;
}

// ---------------------------------------------------------------- covariance / G
// dL/dC of G = V diag(d) V^T, d_i = cof / s_i, s_i = max(l_i, lmax/4),
// cof = h_inv cbrt(s_1 s_2 s_3).
template <class T>
__device__ void g_to_c(const T V[3][3], const T l[3], float h_inv, const float gG[9], T gC[3][3])
{
    T s[3], Jd[3];  // s and which eigenvalue each clamped s follows
    int imax = 0;
    T lmax = fabs(l[0]);
    for (int i = 1; i < 3; ++i)
        if (fabs(l[i]) > lmax) {
            lmax = fabs(l[i]);
            imax = i;
        }
    const T lo = lmax / T(4);
    bool clamped[3];
    for (int i = 0; i < 3; ++i) {
        const T li = fabs(l[i]);
        clamped[i] = li < lo;
        s[i] = clamped[i] ? lo : li;
        Jd[i] = l[i] < T(0) ? T(-1) : T(1);  // d|l|/dl
    }
    const T cof = T(h_inv) * cbrt(s[0] * s[1] * s[2]);
    T d[3];
    for (int i = 0; i < 3; ++i) d[i] = cof / s[i];
    // P = V^T sym(gG) V
    T gs[3][3];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) gs[i][k] = T(0.5) * (T(gG[3 * i + k]) + T(gG[3 * k + i]));
    T P[3][3];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            T acc = T(0);
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n) acc += V[m][i] * gs[m][n] * V[n][k];
            P[i][k] = acc;
        }
    // ds_i/dl_k (J) and dd_i/dl_k = d_i ((1/3) sum_m J_mk / s_m - J_ik / s_i)
    T J[3][3];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) J[i][k] = T(0);
    for (int i = 0; i < 3; ++i) {
        if (clamped[i]) J[i][imax] = Jd[imax] / T(4);
        else J[i][i] = Jd[i];
    }
    T gl[3] = {T(0), T(0), T(0)};
    for (int k = 0; k < 3; ++k) {
        T third = T(0);
        for (int m = 0; m < 3; ++m) third += J[m][k] / s[m];
        third /= T(3);
        for (int i = 0; i < 3; ++i) gl[k] += P[i][i] * d[i] * (third - J[i][k] / s[i]);
    }
    // M = diag(gl) + K o P_offdiag, K_ik = (d_i - d_k) / (l_i - l_k)
    T M[3][3];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            if (i == k) {
                M[i][k] = gl[i];
                continue;
            }
            // divided difference (d_i - d_k) / (l_i - l_k) with d = cof / s:
            // unclamped pairs (s = l > 0) reduce to -cof / (l_i l_k) exactly,
            // which avoids the cancellation of near-degenerate eigenvalues
            T K;
            if (!clamped[i] && !clamped[k]) {
                K = -cof / (s[i] * s[k]);
            } else if (clamped[i] && clamped[k]) {
                K = T(0);
            } else {
                const T dl = l[i] - l[k];
                K = dl != T(0) ? cof * (s[k] - s[i]) / (s[i] * s[k] * dl) : T(0);
            }
            M[i][k] = K * P[i][k];
        }
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            T acc = T(0);
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n) acc += V[i][m] * M[m][n] * V[k][n];
            gC[i][k] = acc;
        }
}

// Calls fn(i, q) for the sorted particles of each lane's cell window (rows of
// x-adjacent cells merged).  Every lane of the warp calls it; lanes with
// active = false take no particles.  A warp whose active windows span at
// most 4 cells per axis walks their union together, 32 particles staged in
// sq at a time (one load per particle for the whole warp); the caller sets
// coop only when every particle the union adds fails each lane's own range
// test, so each lane still sees exactly the particles that matter to it.
// Staged particles beyond r of the box of the active lanes' centres (cx,
// cy, cz) are dropped (they fail every lane's range test); the others keep
// their order, their index rides in the staged w.
template <class Fn>
__device__ __forceinline__ void walk_windows(const Window& w, bool active, bool coop, const Grid& sp,
                                             const uint2* __restrict__ ranges, const float4* __restrict__ sorted,
                                             float4* sq, float cx, float cy, float cz, float r, Fn fn)
{
    const int lane = threadIdx.x & 31;
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
    int ulo[3], uhi[3];
    bool compact = coop;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ulo[a] = (int)__reduce_min_sync(0xffffffffu, active ? (unsigned)w.lo[a] : 0x7fffffffu);
        uhi[a] = (int)__reduce_max_sync(0xffffffffu, active ? (unsigned)(w.hi[a] + 1) : 0u) - 1;
        compact = compact && uhi[a] - ulo[a] <= 3;
    }
    if (compact) {
        const WarpBox box = warp_box(active, cx, cy, cz, r);
        for (int zz = ulo[2]; zz <= uhi[2]; ++zz)
            for (int yy = ulo[1]; yy <= uhi[1]; ++yy) {
                uint32_t beg, end;
                row_range(ulo[0], uhi[0], yy, zz, beg, end);
                for (uint32_t b = beg; b < end; b += 32) {
                    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                    bool keep = false;
                    if (b + lane < end) {
                        q = __ldg(&sorted[b + lane]);
                        keep = box.keeps(q);
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, keep);
                    if (keep) sq[__popc(m & ((1u << lane) - 1u))] = make_float4(q.x, q.y, q.z, __uint_as_float(b + lane));
                    __syncwarp();
                    const uint32_t cnt = __popc(m);
                    if (active)
                        for (uint32_t k = 0; k < cnt; ++k) {
                            const float4 e = sq[k];
                            fn(__float_as_uint(e.w), e);
                        }
                    __syncwarp();
                }
            }
    } else if (active) {
        for (int zz = w.lo[2]; zz <= w.hi[2]; ++zz)
            for (int yy = w.lo[1]; yy <= w.hi[1]; ++yy) {
                uint32_t beg, end;
                row_range(w.lo[0], w.hi[0], yy, zz, beg, end);
                for (uint32_t i = beg; i < end; ++i) fn(i, __ldg(&sorted[i]));
            }
    }
}

// Blocks of two warps (at the registers of 3 blocks of 256 threads per SM):
// a warp without work exits at once, and a small block gives its registers
// back as soon as its two warps are done.
constexpr int kCovBT = 64;

__global__ void __launch_bounds__(kCovBT, 12) k_cov_backward(BwdArgs a, CovArgs f)
{
    __shared__ float4 s_q[kCovBT];  // 32 staged particles per warp
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < f.n;
    float4 gmo = make_float4(0.f, 0.f, 0.f, 0.f);
    float gG[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool act = false;
    float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = c0;
    if (valid) {
        const float4 gr0 = a.gG[3ull * t], gr1 = a.gG[3ull * t + 1], gr2 = a.gG[3ull * t + 2];
        const float g9[9] = {gr0.x, gr0.y, gr0.z, gr1.x, gr1.y, gr1.z, gr2.x, gr2.y, gr2.z};
        bool any = false;
        for (int k = 0; k < 9; ++k) {
            gG[k] = g9[k];
            any = any || g9[k] != 0.f;
        }
        // only involved particles with a non-zero dL/dG whose G used their
        // covariance have work; the forward kept the normalised covariance and
        // its weight sum (k_cov; flag 0: too few neighbours)
        if (any && f.invol[f.skeys[t]] != 0) {
            c0 = f.crec[2ull * t];
            c1 = f.crec[2ull * t + 1];
            act = c1.w != 0.f;
        }
    }
    if (__all_sync(0xffffffffu, !act)) {
        if (valid) a.gmean[t] = gmo;
        return;
    }
    const float4 p = act ? f.sorted[t] : make_float4(0.f, 0.f, 0.f, 1.f);
    const float4 m = act ? f.mean[t] : p;
    const Window w = narrow(window(cell1(p.x, f.sp.min[0], f.sp.cs), cell1(p.y, f.sp.min[1], f.sp.cs),
                                   cell1(p.z, f.sp.min[2], f.sp.cs), 2, f.sp),
                            m.x, m.y, m.z, cull_radius(f.R, f.sp.cs), f.sp);
    float gA[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float gW = 0.f;
    if (act) {
        const float W = c1.z, iw = 1.0f / W;
        float C[3][3] = {{c0.x, c0.y, c0.z}, {c0.y, c0.w, c1.x}, {c0.z, c1.x, c1.y}};
        float C0[3][3];
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) C0[i][k] = C[i][k];
        float lv[3], V[3][3], gC[3][3];
        sym_eig3<float>(C, lv, V);
        const float smax = fmaxf(fabsf(lv[0]), fmaxf(fabsf(lv[1]), fabsf(lv[2])));
        const float smin = fminf(fabsf(lv[0]), fminf(fabsf(lv[1]), fabsf(lv[2])));
        if (!(smin > 0.f) || smax > 1e4f * smin) {
            double Cd[3][3], ld[3], Vd[3][3], gCd[3][3];
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) Cd[i][k] = C0[i][k];
            sym_eig3<double>(Cd, ld, Vd);
            g_to_c<double>(Vd, ld, f.h_inv, gG, gCd);
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) gC[i][k] = (float)gCd[i][k];
        } else {
            g_to_c<float>(V, lv, f.h_inv, gG, gC);
        }
        // C = A / W: dL/dA = gC / W, dL/dW = -<gC, C> / W
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) gW -= gC[i][k] * C0[i][k];
        gW *= iw;
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) gA[i][k] = gC[i][k] * iw;
    }
    const float R = f.R, invR = 1.0f / R, invR3 = invR * invR * invR;
    float gmx = 0.f, gmy = 0.f, gmz = 0.f;
    walk_windows(w, act, f.coop_ok != 0, f.sp, f.ranges, f.sorted, s_q + (threadIdx.x & ~31u), m.x, m.y, m.z,
                 cull_radius(R, f.sp.cs), [&](uint32_t i, const float4& q) {
        const float vx = __fsub_rn(q.x, m.x), vy = __fsub_rn(q.y, m.y), vz = __fsub_rn(q.z, m.z);
        const float d2 = dot3_rn(vx, vy, vz);
        if (!(d2 < f.R_lt2)) return;  // the forward's weight test (d < R), exactly
        const float d = d2 > 0.f ? d2 * rsqrtf(d2) : 0.f;  // the gradient needs no correctly rounded root
        const float s = d * invR;
        const float wt = 1.0f - s * s * s;
        const float Avx = gA[0][0] * vx + gA[0][1] * vy + gA[0][2] * vz;
        const float Avy = gA[1][0] * vx + gA[1][1] * vy + gA[1][2] * vz;
        const float Avz = gA[2][0] * vx + gA[2][1] * vy + gA[2][2] * vz;
        const float vAv = vx * Avx + vy * Avy + vz * Avz;
        // d w / d v = -3 d v / R^3
        const float kw = (vAv + gW) * (-3.0f * d * invR3);
        const float gx = 2.f * wt * Avx + kw * vx, gy = 2.f * wt * Avy + kw * vy, gz = 2.f * wt * Avz + kw * vz;
        atomicAdd(a.gx + i, make_float4(gx, gy, gz, 0.f));
        gmx -= gx;
        gmy -= gy;
        gmz -= gz;
    });
    if (act) gmo = make_float4(gmx, gmy, gmz, 0.f);
    if (valid) a.gmean[t] = gmo;
}

// ---------------------------------------------------------------- smoothing
__global__ void k_smooth_backward(BwdArgs a, const float4* sorted, const float4* mean, const uint2* ranges, Grid sp,
                                  uint32_t n, float R, float R_lt2, int coop_ok, float lambda)
{
    __shared__ float4 s_q[kT];  // 32 staged particles per warp
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < n;
    float4 gs = make_float4(0.f, 0.f, 0.f, 0.f), gmc = gs;
    if (valid) {
        gs = a.gsmooth[t];
        gmc = a.gmean[t];
    }
    const float gmx = lambda * gs.x + gmc.x, gmy = lambda * gs.y + gmc.y, gmz = lambda * gs.z + gmc.z;
    float gix = (1.0f - lambda) * gs.x, giy = (1.0f - lambda) * gs.y, giz = (1.0f - lambda) * gs.z;
    const bool act = valid && (gmx != 0.f || gmy != 0.f || gmz != 0.f);
    if (__any_sync(0xffffffffu, act)) {
        const float4 p = act ? sorted[t] : make_float4(0.f, 0.f, 0.f, 1.f);
        const float4 m = act ? mean[t] : make_float4(0.f, 0.f, 0.f, 1.f);  // m.w: the forward's weight sum W
        const Window w = narrow(window(cell1(p.x, sp.min[0], sp.cs), cell1(p.y, sp.min[1], sp.cs),
                                       cell1(p.z, sp.min[2], sp.cs), 2, sp),
                                p.x, p.y, p.z, cull_radius(R, sp.cs), sp);
        const float iw = 1.0f / m.w;
        const float gnx = gmx * iw, gny = gmy * iw, gnz = gmz * iw;
        const float invR = 1.0f / R, invR3 = invR * invR * invR;
        walk_windows(w, act, coop_ok != 0, sp, ranges, sorted, s_q + (threadIdx.x & ~31u), p.x, p.y, p.z,
                     cull_radius(R, sp.cs),
                     [&](uint32_t i, const float4& q) {
            // the forward's neighbour decision, exactly
            const float d2 = dot3_rn(__fsub_rn(p.x, q.x), __fsub_rn(p.y, q.y), __fsub_rn(p.z, q.z));
            if (!(d2 < R_lt2)) return;
            const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
            const float d = d2 > 0.f ? d2 * rsqrtf(d2) : 0.f;
            const float s = d * invR;
            const float wt = 1.0f - s * s * s;
            // mean = sum w x / W: dL/dx_j += w gN, dL/dw = <gN, x_j - mean>
            const float gw = gnx * (q.x - m.x) + gny * (q.y - m.y) + gnz * (q.z - m.z);
            // dw/dd (x_i - x_j) / d = -3 d / R^3 (x_i - x_j)
            const float k = gw * (-3.0f * d * invR3);
            const float ex = k * dx, ey = k * dy, ez = k * dz;
            gix += ex;
            giy += ey;
            giz += ez;
            atomicAdd(a.gx + i, make_float4(wt * gnx - ex, wt * gny - ey, wt * gnz - ez, 0.f));
        });
    }
    if (valid) atomicAdd(a.gx + t, make_float4(gix, giy, giz, 0.f));
}

__global__ void k_unsort(const float4* gx, const uint32_t* perm, uint32_t n, float* out)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 g = gx[k];
    const uint32_t s = perm[k];
    out[3ull * s] = g.x;
    out[3ull * s + 1] = g.y;
    out[3ull * s + 2] = g.z;
}

inline unsigned nblk(uint64_t n) { return (unsigned)std::max<uint64_t>(1, (n + kT - 1) / kT); }

}  // namespace

void launch_backward(const KernelCtx& c, const BwdArgs& a, const CovArgs* cov, const Counters* ctr, int method,
                     float lambda, float R, float* radius_grad_dev, float* out_grad_xyz)
{
    const unsigned pb = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((a.cap_valid + kT - 1) / kT,
                                                                          (uint64_t)c.num_sms * 16));
    k_mc_backward<<<pb, kT, 0, c.stream>>>(a, ctr);
    const unsigned bb = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((a.cap_band + kT - 1) / kT,
                                                                          (uint64_t)c.num_sms * 16));
    k_mark_keys<<<bb, kT, 0, c.stream>>>(a, ctr);
    g_launches += 2;
    if (method == FSR_METHOD_YU13) {
        AnisoBwdArgs fb{};
        fb.sp = a.sp;
        fb.sc = a.sc;
        fb.band = a.band;
        fb.smoothed = a.smoothed;
        fb.grec = a.grec;
        fb.qrec = a.qrec;
        fb.ranges = a.ranges;
        fb.invol = a.invol;
        fb.cell_rmax = a.cell_rmax;
        fb.gphi = a.gphi;
        fb.glist = a.glist;
        fb.gsmooth = a.gsmooth;
        fb.gG = a.gG;
        fb.sigma = a.sigma;
        fb.cap = a.cap_band;
        if (launch_field_aniso_backward_grouped(c, fb, a.ratio, ctr)) {
            k_det_term<<<nblk(a.n), kT, 0, c.stream>>>(a);
        } else {
            k_field_backward_aniso<<<nblk(a.n), kT, 0, c.stream>>>(a);
        }
        k_cov_backward<<<(unsigned)std::max<uint64_t>(1, (a.n + kCovBT - 1) / kCovBT), kCovBT, 0, c.stream>>>(a, *cov);
        // warps may walk the union of their windows when the cull radius stays below 2 cells
        const int smooth_coop = (R * 1.0001f + 1e-4f * cov->sp.cs) < 2.0f * cov->sp.cs * 0.9999f ? 1 : 0;
        k_smooth_backward<<<nblk(a.n), kT, 0, c.stream>>>(a, cov->sorted, cov->mean, cov->ranges, cov->sp, a.n, R,
                                                           cov->R_lt2, smooth_coop, lambda);
        g_launches += 3;
    } else if (method == FSR_METHOD_TC01) {
        if (!launch_field_iso_backward_grouped(c, a, true, ctr)) {
            k_field_backward_iso<true><<<nblk(a.n), kT, 0, c.stream>>>(a);
            ++g_launches;
        }
    } else {
        if (!launch_field_iso_backward_grouped(c, a, false, ctr)) {
            k_field_backward_iso<false><<<nblk(a.n), kT, 0, c.stream>>>(a);
            ++g_launches;
        }
        if (radius_grad_dev) {
            k_radius_grad<<<bb, kT, 0, c.stream>>>(a, ctr, radius_grad_dev);
            ++g_launches;
        }
    }
    k_unsort<<<nblk(a.n), kT, 0, c.stream>>>(a.gx, a.perm, a.n, out_grad_xyz);
    ++g_launches;
}

}  // namespace fsr
