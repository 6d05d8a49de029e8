// Shared device-side definitions of the reconstruction kernels.
//
// Arithmetic policy.  Every value that feeds a discrete decision - a cell
// index, a grid-vertex position, a band-membership or neighbour-count test,
// a surface-particle test - is computed with explicitly rounded FP32
// operations (__fadd_rn & co.) in the reference's operation order, so it
// cannot be contracted into an FMA and the decision matches the reference
// source evaluated in IEEE FP32 bit for bit.  Continuous accumulations that
// only feed the field value (kernel sums, covariances) are free to use FMA
// and any summation order; they are checked against the FP64 oracle within
// the stated tolerance.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mc_tables.h"

namespace fsr {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;

// Uniform grid (GridInfo, Defines.h:62-68, without the unused maxPos).
struct Grid {
    float min[3];
    float cs;
    uint32_t res[3];
    uint32_t pad;
};

// Device-resident frame counters: sizes that later stages read, plus error
// and capacity-overflow flags.  Filled by the kernels, read once per frame.
struct Counters {
    uint32_t n_band;         // B
    uint32_t n_valid;        // Q
    uint32_t n_mesh_verts;   // 3T
    uint32_t n_surface;      // surface particles
    uint32_t n_involved;     // Yu13 involved particles
    uint32_t n_fp64;         // eigen solves redone in FP64
    uint32_t out_of_grid;    // particles outside the grid (error)
    uint32_t overflow;       // bit 0: band, bit 1: valid cubes, bit 2: mesh vertices
    uint32_t need_band;      // sizes wanted when an overflow happened
    uint32_t need_valid;
    uint32_t need_mesh;
    uint32_t work_field;     // next window group of the anisotropic field (dynamic scheduling)
    uint32_t work_adjoint;   // the same for its adjoint
    uint32_t n_weld;         // welded mesh vertices (FSR_FLAG_WELD)
    uint32_t n_groups;       // window groups holding band vertices (the field's work list)
    uint32_t pad[1];
};

// Rank directory over the band bitset: rank(v) = number of band vertices
// with a smaller id, valid when v itself is in the band.
struct BandView {
    const uint32_t* bits;    // V bits
    const uint32_t* prefix;  // exclusive prefix of popcount per 32-bit word
    const float* phi;        // field per band vertex, in rank order
};

// Marching-cubes tables in constant memory.
struct McConst {
    uint64_t tri[256];
    uint16_t eflags[256];
    uint8_t nverts[256];
};

#if defined(__CUDACC__)
__device__ __forceinline__ uint32_t lin3(uint32_t x, uint32_t y, uint32_t z, const Grid g)
{
    return z * g.res[0] * g.res[1] + y * g.res[0] + x;
}

__device__ __forceinline__ void unlin3(uint32_t i, const Grid& g, uint32_t& x, uint32_t& y, uint32_t& z)
{
    const uint32_t xy = g.res[0] * g.res[1];
    z = i / xy;
    const uint32_t m = i - z * xy;
    y = m / g.res[0];
    x = m - y * g.res[0];
}

// getIndex3D (ReconstructionCUDA.cuh:354-358): trunc((p - min) / cs).
__device__ __forceinline__ int cell1(float p, float mn, float cs)
{
    return __float2int_rz(__fdiv_rn(__fsub_rn(p, mn), cs));
}

// getVertexPos (ReconstructionCUDA.cuh:366-370): float(i) * cs + min, with
// the product rounded before the sum.
__device__ __forceinline__ float vpos1(uint32_t i, float mn, float cs)
{
    return __fadd_rn(__fmul_rn(__uint2float_rn(i), cs), mn);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// dot(d, d) of helper_math: (x*x + y*y) + z*z, each product rounded.
__device__ __forceinline__ float dot3_rn(float x, float y, float z)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}

// Cells c-ext .. c+ext clamped to the grid (scalar members: no local arrays).
struct Window {
    int lo[3], hi[3];
};

__device__ __forceinline__ Window window(int cx, int cy, int cz, int ext, const Grid g)
{
    Window w;
    w.lo[0] = clampi(cx - ext, 0, (int)g.res[0] - 1);
    w.lo[1] = clampi(cy - ext, 0, (int)g.res[1] - 1);
    w.lo[2] = clampi(cz - ext, 0, (int)g.res[2] - 1);
    w.hi[0] = clampi(cx + ext, 0, (int)g.res[0] - 1);
    w.hi[1] = clampi(cy + ext, 0, (int)g.res[1] - 1);
    w.hi[2] = clampi(cz + ext, 0, (int)g.res[2] - 1);
    return w;
}

// Narrows a window to the cells whose extent on each axis comes within r of
// point p.  Callers pass r with a relative margin, so every particle a
// skipped cell holds lies farther than the unmargined radius on some axis
// even after the roundings of its cell index and of the distance: terms that
// contribute exactly zero are the only ones skipped.
__device__ __forceinline__ Window narrow(const Window& w, float px, float py, float pz, float r, const Grid g)
{
    Window o;
    const float inv = 1.0f / g.cs;
    o.lo[0] = max(w.lo[0], __float2int_rd((px - r - g.min[0]) * inv));
    o.lo[1] = max(w.lo[1], __float2int_rd((py - r - g.min[1]) * inv));
    o.lo[2] = max(w.lo[2], __float2int_rd((pz - r - g.min[2]) * inv));
    o.hi[0] = min(w.hi[0], __float2int_rd((px + r - g.min[0]) * inv));
    o.hi[1] = min(w.hi[1], __float2int_rd((py + r - g.min[1]) * inv));
    o.hi[2] = min(w.hi[2], __float2int_rd((pz + r - g.min[2]) * inv));
    return o;
}

// Margin applied to culling radii: relative 1e-4 plus 1e-4 of a cell.
__device__ __forceinline__ float cull_radius(float r, float cs) { return r * 1.0001f + 1e-4f * cs; }

// Box of the warp's active centres grown by r: a candidate outside it lies
// beyond r of every active lane's centre.
struct WarpBox {
    float lo[3], hi[3], r, r2;
    __device__ __forceinline__ bool holds(const float4& q) const
    {
        return q.x >= lo[0] && q.x <= hi[0] && q.y >= lo[1] && q.y <= hi[1] && q.z >= lo[2] && q.z <= hi[2];
    }
    // q lies within r of the centres' box itself: the corners of the grown
    // box are rounded off (about 30 % fewer candidates for a half-cell box
    // and r near one cell).  The centres' box is recovered as lo + r and
    // hi - r; r2 is (r + m)^2 with m four units in the last place of the
    // box's largest coordinate, above the roundings of that recovery and of
    // the distance, so a candidate within r of some centre is never dropped.
    __device__ __forceinline__ bool reaches(const float4& q) const
    {
        const float gx = fmaxf(0.f, fmaxf((lo[0] + r) - q.x, q.x - (hi[0] - r)));
        const float gy = fmaxf(0.f, fmaxf((lo[1] + r) - q.y, q.y - (hi[1] - r)));
        const float gz = fmaxf(0.f, fmaxf((lo[2] + r) - q.z, q.z - (hi[2] - r)));
        return fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < r2;
    }
    __device__ __forceinline__ bool keeps(const float4& q) const { return holds(q) && reaches(q); }
};

__device__ __forceinline__ WarpBox warp_box(bool active, float x, float y, float z, float r)
{
    WarpBox b;
    float lo[3] = {active ? x : 3.0e38f, active ? y : 3.0e38f, active ? z : 3.0e38f};
    float hi[3] = {active ? x : -3.0e38f, active ? y : -3.0e38f, active ? z : -3.0e38f};
    float big = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
        b.lo[a] = lo[a] - r;
        b.hi[a] = hi[a] + r;
        big = fmaxf(big, fmaxf(fabsf(b.lo[a]), fabsf(b.hi[a])));
    }
    b.r = r;
    const float m = r + 4.0f * 1.1920929e-7f * big;  // 2^-23: one unit in the last place per unit of magnitude
    b.r2 = m * m;
    return b;
}

// float(k * (double)x * (double)x) for k < 0 and x in (0, 1], the colour
// field's spiky gradient as the reference evaluates it in double
// (extractionOfSurfaceParticlesUsingColorField, cu:909-971), computed in
// FP32 (this GPU's FP64 rate is a small fraction of its FP32 rate).  |k| is
// split on the host into khi + klo (floats); |k| x^2 is formed as a float
// pair with exact products (FMA) to within 2^-44 relative, and rounded to
// float; the reference's value, within 2^-52 of the exact product, rounds to
// the same float unless the exact product lies near a rounding midpoint.
// Those cases (the pair's value within 2^-40 of a midpoint, about one
// evaluation in 2^19) take the double expression itself.  fsr_check_spiky_grad
// compares it with the double expression for every float x in (0, 1].
// The double expression, out of line so that the compiler keeps it behind a
// branch instead of evaluating it on every call.
static __device__ __noinline__ float spiky_grad_double(float x, double k)
{
    return __double2float_rn(__dmul_rn(__dmul_rn(k, (double)x), (double)x));
}

__device__ __forceinline__ float spiky_grad(float x, float khi, float klo, double k)
{
    const float ph = __fmul_rn(khi, x);
    const float pl = fmaf(khi, x, -ph);       // khi x = ph + pl exactly
    const float b = fmaf(klo, x, pl);         // |k| x = ph + b (1 + 2^-46)
    const float qh = __fmul_rn(ph, x);
    const float ql = fmaf(ph, x, -qh);        // ph x = qh + ql exactly
    const float l = fmaf(b, x, ql);           // |k| x^2 = qh + l (1 + 2^-45)
    const float r = __fadd_rn(qh, l);
    const float bb = __fsub_rn(r, qh);        // two-sum: err = qh + l - r exactly
    const float err = __fadd_rn(__fsub_rn(qh, __fsub_rn(r, bb)), __fsub_rn(l, bb));
    const float up = __fsub_rn(__int_as_float(__float_as_int(r) + 1), r);  // the ulps above and below r
    const float dn = __fsub_rn(r, __int_as_float(__float_as_int(r) - 1));
    const float margin = r * 0x1p-40f;
    if (fmaf(0.5f, up, -err) <= margin || fmaf(0.5f, dn, err) <= margin) return spiky_grad_double(x, k);
    return -r;
}

// a / b correctly rounded (the same float as __fdiv_rn(a, b)) for a >= 0,
// b > 0, given rb = RN(1 / b) computed once on the host.  Markstein's
// theorem (P. Markstein, IBM J. Res. Dev. 34(1), 1990; Muller et al.,
// Handbook of Floating-Point Arithmetic, "division with an FMA"): with y
// within half an ulp of 1/b and q within one ulp of a/b, the remainder
// r = a - b q is exact under an FMA and RN(q + r y) = RN(a / b), as long as
// nothing underflows; tiny positive a (below 2^-64) take the IEEE division.
// Three instructions instead of the IEEE division's sequence;
// fsr_check_division verifies it against __fdiv_rn for every float a in
// [0, 1.01 b].
__device__ __forceinline__ float div_exact(float a, float b, float rb)
{
    if (a < 0x1p-64f && a > 0.0f) return __fdiv_rn(a, b);
    const float q = __fmul_rn(a, rb);
    const float r = fmaf(-q, b, a);
    return fmaf(r, rb, q);
}

__device__ __forceinline__ bool band_has(const BandView& b, uint32_t v)
{
    return (__ldg(b.bits + (v >> 5)) >> (v & 31u)) & 1u;
}

__device__ __forceinline__ uint32_t band_rank(const BandView& b, uint32_t v)
{
    const uint32_t w = __ldg(b.bits + (v >> 5));
    return __ldg(b.prefix + (v >> 5)) + __popc(w & ((1u << (v & 31u)) - 1u));
}

// First grid-vertex index along AXIS whose FP32 cell index (getIndex3D of
// the vertex position) is >= c.  The cell index is non-decreasing along the
// axis; the boundary lies within a vertex or two of c * ratio.
template <int AXIS>
__device__ __forceinline__ int first_vertex(int c, const Grid& sc, const Grid& sp, uint32_t ratio)
{
    int x = max(0, c * (int)ratio - 1);
    const int nres = (int)sc.res[AXIS];
    if (x > nres) x = nres;
    while (x > 0 && cell1(vpos1(x - 1, sc.min[AXIS], sc.cs), sp.min[AXIS], sp.cs) >= c) --x;
    while (x < nres && cell1(vpos1(x, sc.min[AXIS], sc.cs), sp.min[AXIS], sp.cs) < c) ++x;
    return x;
}

#endif  // __CUDACC__

}  // namespace fsr
