// Anisotropic field, grouped by window (computationOfScalarFieldGrid,
// ReconstructionCUDA.cu:830-906).
//
// A band vertex's candidate particles are the particles of the +-2 cells
// around the spatial cell its FP32 position falls in; every vertex that
// falls in the same cell has the same window.  Along each axis that cell
// index is a non-decreasing function of the vertex index, so the vertices
// of one cell form an index box, found exactly without sorting.  One warp
// handles one such group (or one z slab of it, for frames with few groups),
// taken from a work counter:
//   1. it lists the group's band vertices row by row from the bitset, with
//      their rank in the band, in passes of up to 256 vertices ordered into
//      eight brick tiles of 32;
//   2. it lists the window's candidate cells, dropping involved cells that
//      lie beyond the reach (largest support radius + smoothing shift) of all
//      their particles from the group's vertex box;
//   3. it streams the involved candidates 32 at a time (one record per lane,
//      kept in shared memory when its support reaches the pass's box); per
//      tile, the candidates that reach the tile are listed two to a pair
//      block and each lane evaluates one block per step for its vertex with
//      packed FP32x2 operations.
// Particles of non-involved cells use the unscaled kernel (cuh:312-322),
// G = I with support 1: their part of each vertex's sum is the group's
// moment polynomial where it applies, else they are streamed as well.  Only
// terms that are exactly zero are skipped; the summation order is the
// candidate order, the same for every vertex, so results are deterministic.
#include "kernels.h"
#include "backward.h"

#include <algorithm>

namespace fsr {
namespace {

constexpr int kBT = 256;            // threads per block
constexpr int kMaxCells = 125;      // 5 x 5 x 5 window

struct GroupArgs {
    Grid sp, sc;
    BandView band;
    const float4* grec;
    const float4* qrec;  // per involved particle: (x~, r2max) (M00, 2M01, 2M02, coef) (M11, 2M12, M22, 0)
    const float4* smoothed;
    const uint32_t* glist;  // groups holding band vertices
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

// Work items of the forward field kernels: a frame with few window groups
// (a small frame) would leave most SMs idle with one warp per group, so each
// group's vertex box is then cut into S slabs along z, each a work item of
// its own (a vertex lies in one slab; a slab is listed, culled and summed
// like a group).  S depends only on the number of groups, so a frame's
// results do not depend on the launch shape.
constexpr uint32_t kSlabTarget = 8192;  // work items wanted (measured: 4096 and 8 slabs at most, 12-16 % slower on 32k frames)
constexpr uint32_t kSlabMax = 16;
__device__ __forceinline__ uint32_t field_slabs(uint32_t ngroups)
{
    return ngroups >= kSlabTarget ? 1u : min(kSlabMax, (kSlabTarget + ngroups - 1) / max(ngroups, 1u));
}
// Restricts the box [lo, hi) to slab `part` of S along z; false when empty.
__device__ __forceinline__ bool slab_box(uint32_t part, uint32_t S, int lo[3], int hi[3])
{
    if (S == 1) return true;
    const uint32_t nz = (uint32_t)(hi[2] - lo[2]);
    const int z0 = lo[2] + (int)(nz * part / S), z1 = lo[2] + (int)(nz * (part + 1) / S);
    if (z0 >= z1) return false;
    lo[2] = z0;
    hi[2] = z1;
    return true;
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
__device__ __forceinline__ uint32_t candidate(uint32_t j, const CandTables& t, int* cell, int ncells = kMaxCells)
{
    int lo = 0, hi = ncells;  // find k with cpre[k] <= j < cpre[k+1]
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

// ---------------------------------------------------------------- forward
constexpr int kFT = 128;                 // threads per block of the forward kernel
#ifndef FSR_FIELD_MIN_BLOCKS
#define FSR_FIELD_MIN_BLOCKS 6               // blocks per SM of the anisotropic field (80 registers)
#endif
constexpr int kFWarps = kFT / 32;
constexpr int kPassTiles = 8;            // 32-vertex tiles per pass (sums kept per lane in the warp's slice)
constexpr int kPassVerts = 32 * kPassTiles;
constexpr int kMoments = 35;             // moments of the unscaled kernel's polynomial (unscaled_sum)
constexpr int kPairF4 = 5;               // float4 per pair block of listed candidates (list_pair_record)

// Per-warp shared memory of the forward kernel.
struct WarpSlice {
    float4 rec[80];              // the current chunk's candidates: 5 float2 per lane (involved, stage_record),
                                 // a float4 per lane (the others)
    float4 lst[16 * kPairF4];    // one tile's involved candidates in lane order, two to a pair block
    uint32_t vloc[kPassVerts];   // the pass's band vertices: index in the group's box (vert_loc)
    uint32_t vrank[kPassVerts];  // and band rank
    float4 box[2 * kPassTiles];  // per tile: lo, hi
    float psum[kPassTiles][32];  // per tile and lane: sum over the involved candidates
    float usum[kPassTiles][32];  // and over the non-involved ones
    uint16_t order[kPassVerts];  // the pass's vertices in brick order (tile t: entries 32t .. 32t+31)
    float mom[kMoments];         // moments of the group's non-involved candidates (unscaled_moments)
    uint32_t use_mom;            // the moment form applies to this group
    uint32_t cstart[128];
    uint32_t cpre[kMaxCells + 1];
    uint32_t cinv[128];
    uint32_t ncells;             // entries of the candidate tables
    uint32_t total_inv;          // candidates of involved cells (they come first)
    uint32_t ninv_cells;         // and the number of those cells
};

// The window cells of candidates cb .. cb + 31 of a sweep through the
// tables, one per lane, from the table boundaries that fall inside the
// chunk (one shared load and a warp OR instead of a binary search per
// lane).  k0 is a cell with cpre[k0] <= cb < cpre[k0 + 1] on entry (the
// sweep's first cell, or the value the previous chunk left) and is advanced
// to the cell of cb + 31.  Every lane calls it; the cell of a lane whose
// candidate lies at or beyond the sweep's end is not used.
__device__ __forceinline__ int chunk_cell(uint32_t cb, int lane, const uint32_t* cpre, uint32_t ncells, uint32_t& k0)
{
    const uint32_t k = k0 + 1u + (uint32_t)lane;
    uint32_t bit = 0;
    if (k <= ncells) {
        const uint32_t d = cpre[k] - cb;  // cpre[k] >= cpre[k0 + 1] > cb
        if (d < 32u) bit = 1u << d;
    }
    const uint32_t bm = __reduce_or_sync(0xffffffffu, bit);
    const int cell = (int)(k0 + (uint32_t)__popc(bm & (0xffffffffu >> (31 - lane))));
    k0 += (uint32_t)__popc(bm);
    return cell;
}

// Warp-level version of group_candidates: the same cells, listed with the
// involved cells first and the other non-empty cells after them (each part
// in window order); only non-empty kept cells get an entry.
__device__ uint32_t warp_candidates(const Grid& sp, const uint2* __restrict__ ranges,
                                    const uint8_t* __restrict__ invol, const float* __restrict__ reach,
                                    const int c[3], const float b0[3], const float b1[3], WarpSlice& w)
{
    const int lane = threadIdx.x & 31;
    const int lx = clampi(c[0] - 2, 0, (int)sp.res[0] - 1), hx = clampi(c[0] + 2, 0, (int)sp.res[0] - 1);
    const int ly = clampi(c[1] - 2, 0, (int)sp.res[1] - 1), hy = clampi(c[1] + 2, 0, (int)sp.res[1] - 1);
    const int lz = clampi(c[2] - 2, 0, (int)sp.res[2] - 1), hz = clampi(c[2] + 2, 0, (int)sp.res[2] - 1);
    uint32_t st4[4], cnt4[4], inv4[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int k = 32 * r + lane;
        uint32_t cnt = 0, st = 0, inv = 0;
        if (k < kMaxCells) {
            const int xx = lx + k % 5, yy = ly + (k / 5) % 5, zz = lz + k / 25;
            if (xx <= hx && yy <= hy && zz <= hz) {
                const uint32_t cell = lin3(xx, yy, zz, sp);
                const uint2 rg = __ldg(&ranges[cell]);
                if (rg.x != kEmpty) {
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
                        st = rg.x;
                        cnt = rg.y - rg.x;
                    }
                }
            }
        }
        st4[r] = st;
        cnt4[r] = cnt;
        inv4[r] = inv;
    }
    // two sweeps: involved cells, then the others; entries and prefix sums
    // are appended in window order within each sweep
    uint32_t running = 0, slot = 0;
#pragma unroll
    for (int part = 0; part < 2; ++part) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const bool take = cnt4[r] > 0 && (inv4[r] != 0) == (part == 0);
            const uint32_t m = __ballot_sync(0xffffffffu, take);
            const uint32_t c = take ? cnt4[r] : 0u;
            uint32_t x = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (take) {
                const uint32_t e = slot + __popc(m & ((1u << lane) - 1u));
                w.cstart[e] = st4[r];
                w.cinv[e] = inv4[r];
                w.cpre[e] = running + x - c;
            }
            slot += __popc(m);
            running += __shfl_sync(0xffffffffu, x, 31);
        }
        if (part == 0 && lane == 0) {
            w.total_inv = running;
            w.ninv_cells = slot;
        }
    }
    if (lane == 0) {
        w.cpre[slot] = running;
        w.ncells = slot;
    }
    __syncwarp();
    return running;
}

// A staged involved candidate: 10 floats per lane, as 5 float2
//   (x~, y~) (z~, M00) (2M01, 2M02) (M11, 2M12) (M22, coef)
// (M = G^T G; coef = sigma det(G) m / rho).
__device__ __forceinline__ void stage_record(float2* rec, int lane, float4 r0, float4 m0, float4 m1)
{
    float2* d = rec + 5 * lane;
    d[0] = make_float2(r0.x, r0.y);
    d[1] = make_float2(r0.z, m0.x);
    d[2] = make_float2(m0.y, m0.z);
    d[3] = make_float2(m1.x, m1.y);
    d[4] = make_float2(m1.z, m0.w);
}

// A tile's candidates are listed two to a pair block of 5 float4: entry pos
// of the list in the x (and z) components, entry pos + 1 in y (and w), so
// that each float2 of the block holds one quantity of both candidates and
// feeds one packed FP32x2 operation:
//   (x~, x~') (y~, y~') | (z~, z~') (M00, M00') | (2M01, 2M01') (2M02, 2M02') |
//   (M11, M11') (2M12, 2M12') | (M22, M22') (coef, coef')
__device__ __forceinline__ void list_pair_record(const float2* rec, int lane, float* lst, uint32_t pos)
{
    const float2* src = rec + 5 * lane;
    float* d = lst + (pos >> 1) * (4 * kPairF4) + (pos & 1u);
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        const float2 v = src[c];
        d[4 * c] = v.x;
        d[4 * c + 2] = v.y;
    }
}

// The (1 - q2)^3 terms of both candidates of a pair block for vertex v
// (nv = (-v, -v) per axis): q2 = d^T M d for d = x~ - v, each component
// rounded as the scalar form
//   t1 = fma(M00, dx, fma(2M01, dy, 2M02 dz)),  t2 = fma(M11, dy, 2M12 dz),
//   q2 = fma(dx, t1, fma(dy, t2, dz (M22 dz))),  (1 - q2)^3 = ((1 - q2)^2)(1 - q2)
// (no product feeds a separate sum, so no contraction can change a rounding).
__device__ __forceinline__ void pair_terms(const float4* P, float2 nvx, float2 nvy, float2 nvz, float2& q2,
                                           float2& u3, float2& coef)
{
    const float4 A = P[0], B = P[1], C = P[2], D = P[3], E = P[4];
    const float2 dx = __fadd2_rn(make_float2(A.x, A.y), nvx);
    const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nvy);
    const float2 dz = __fadd2_rn(make_float2(B.x, B.y), nvz);
    float2 t1 = __fmul2_rn(make_float2(C.z, C.w), dz);
    t1 = __ffma2_rn(make_float2(C.x, C.y), dy, t1);
    t1 = __ffma2_rn(make_float2(B.z, B.w), dx, t1);
    float2 t2 = __fmul2_rn(make_float2(D.z, D.w), dz);
    t2 = __ffma2_rn(make_float2(D.x, D.y), dy, t2);
    float2 q = __fmul2_rn(make_float2(E.x, E.y), dz);
    q = __fmul2_rn(dz, q);
    q = __ffma2_rn(dy, t2, q);
    q = __ffma2_rn(dx, t1, q);
    // 1 - q2 as fma(q2, -1, 1): the product is exact, so one rounding, as in
    // the subtraction
    const float2 u = __ffma2_rn(q, make_float2(-1.0f, -1.0f), make_float2(1.0f, 1.0f));
    u3 = __fmul2_rn(__fmul2_rn(u, u), u);
    q2 = q;
    coef = make_float2(E.z, E.w);
}

__device__ __forceinline__ bool reaches(float4 r0, float4 lo, float4 hi)
{
    const float gx = fmaxf(0.f, fmaxf(lo.x - r0.x, r0.x - hi.x));
    const float gy = fmaxf(0.f, fmaxf(lo.y - r0.y, r0.y - hi.y));
    const float gz = fmaxf(0.f, fmaxf(lo.z - r0.z, r0.z - hi.z));
    return fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < r0.w;
}

// A listed vertex is kept as its index in the group's box, 10 bits per axis
// (the box spans at most ratio + 1 <= 1001 vertices per axis); its position
// is the scalar grid's vertex position (getVertexPos, FP32).
__device__ __forceinline__ uint32_t vert_loc(int lx, int ly, int lz)
{
    return (uint32_t)lx | ((uint32_t)ly << 10) | ((uint32_t)lz << 20);
}

__device__ __forceinline__ float4 vert_pos(uint32_t loc, const int lo[3], const Grid& sc)
{
    return make_float4(vpos1(lo[0] + (int)(loc & 1023u), sc.min[0], sc.cs),
                       vpos1(lo[1] + (int)((loc >> 10) & 1023u), sc.min[1], sc.cs),
                       vpos1(lo[2] + (int)(loc >> 20), sc.min[2], sc.cs), 0.f);
}

// The layout of a pass of nv <= kPassVerts listed vertices: the pass's box
// (pl, ph, on every lane), their order in 4 x 4 x 2-vertex bricks (tiles of
// compact bricks instead of runs of rows: a smaller box per tile, fewer
// candidates reaching it; a counting sort by brick, the order within a brick
// is that of the atomics, which changes no result since a vertex's sum does
// not depend on its tile and culling only skips exact zeros), and the box of
// each 32-vertex tile.  hist: kPassVerts words of scratch.
__device__ __forceinline__ void pass_layout(const uint32_t* vloc, const int lo[3], const Grid& sc, uint16_t* order,
                                            uint32_t* hist, float4* box, uint32_t nv, float inv, int lane, float4& pl,
                                            float4& ph)
{
    const uint32_t ntiles = (nv + 31) / 32;
    pl = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f);
    ph = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
    for (uint32_t q = lane; q < nv; q += 32) {
        const float4 v = vert_pos(vloc[q], lo, sc);
        pl.x = fminf(pl.x, v.x); pl.y = fminf(pl.y, v.y); pl.z = fminf(pl.z, v.z);
        ph.x = fmaxf(ph.x, v.x); ph.y = fmaxf(ph.y, v.y); ph.z = fmaxf(ph.z, v.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pl.x = fminf(pl.x, __shfl_xor_sync(0xffffffffu, pl.x, o));
        pl.y = fminf(pl.y, __shfl_xor_sync(0xffffffffu, pl.y, o));
        pl.z = fminf(pl.z, __shfl_xor_sync(0xffffffffu, pl.z, o));
        ph.x = fmaxf(ph.x, __shfl_xor_sync(0xffffffffu, ph.x, o));
        ph.y = fmaxf(ph.y, __shfl_xor_sync(0xffffffffu, ph.y, o));
        ph.z = fmaxf(ph.z, __shfl_xor_sync(0xffffffffu, ph.z, o));
    }
    const int gx = (__float2int_rn((ph.x - pl.x) * inv) >> 2) + 1;
    const int gy = (__float2int_rn((ph.y - pl.y) * inv) >> 2) + 1;
    const int gz = (__float2int_rn((ph.z - pl.z) * inv) >> 1) + 1;
    const int nbins = gx * gy * gz;
    if (nbins <= kPassVerts) {
        for (int b = lane; b < nbins; b += 32) hist[b] = 0u;
        __syncwarp();
        int key[kPassVerts / 32];
        uint32_t slot[kPassVerts / 32];
#pragma unroll
        for (int k = 0; k < kPassVerts / 32; ++k) {
            const uint32_t q = lane + 32 * k;
            key[k] = 0;
            slot[k] = 0;
            if (q < nv) {
                const float4 v = vert_pos(vloc[q], lo, sc);
                const int ix = __float2int_rn((v.x - pl.x) * inv) >> 2;
                const int iy = __float2int_rn((v.y - pl.y) * inv) >> 2;
                const int iz = __float2int_rn((v.z - pl.z) * inv) >> 1;
                key[k] = min(ix, gx - 1) + gx * (min(iy, gy - 1) + gy * min(iz, gz - 1));
                slot[k] = atomicAdd(hist + key[k], 1u);
            }
        }
        __syncwarp();
        // exclusive scan of the bins, lane by lane in blocks of nbins / 32
        const int per = (nbins + 31) / 32;
        uint32_t tot = 0;
        for (int b = lane * per; b < min(nbins, lane * per + per); ++b) tot += hist[b];
        uint32_t x = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        uint32_t run = x - tot;
        __syncwarp();
        for (int b = lane * per; b < min(nbins, lane * per + per); ++b) {
            const uint32_t hcount = hist[b];
            hist[b] = run;
            run += hcount;
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < kPassVerts / 32; ++k) {
            const uint32_t q = lane + 32 * k;
            if (q < nv) order[hist[key[k]] + slot[k]] = (uint16_t)q;
        }
    } else {
        for (uint32_t q = lane; q < nv; q += 32) order[q] = (uint16_t)q;
    }
    __syncwarp();
    if ((uint32_t)lane < ntiles) {
        float4 tl = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f), th = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
        for (uint32_t q = 32 * lane; q < min(nv, 32 * lane + 32); ++q) {
            const float4 v = vert_pos(vloc[order[q]], lo, sc);
            tl.x = fminf(tl.x, v.x); tl.y = fminf(tl.y, v.y); tl.z = fminf(tl.z, v.z);
            th.x = fmaxf(th.x, v.x); th.y = fmaxf(th.y, v.y); th.z = fmaxf(th.z, v.z);
        }
        box[2 * lane] = tl;
        box[2 * lane + 1] = th;
    }
    __syncwarp();
}

// The band vertices of a group's index box [lo, hi), listed into (vloc,
// vrank) by row segments of at most 32 vertices (two bitset
// words), `per` segments per step so that one step adds at most kPassVerts
// vertices; pass(count) runs whenever the next step would not fit, and at
// the end.
template <class PassFn>
__device__ __forceinline__ void list_band_vertices(const Grid& sc, const BandView& band, const int lo[3],
                                                   const int hi[3], uint32_t* vloc, uint32_t* vrank, int lane,
                                                   PassFn&& pass)
{
    const int nx = hi[0] - lo[0], ny = hi[1] - lo[1], nz = hi[2] - lo[2];
    const int nseg = (nx + 31) / 32;
    const int units = ny * nz * nseg;
    const int per = max(1, min(32, kPassVerts / min(nx, 32)));
    int ub = 0;
    while (ub < units) {
        uint32_t count = 0;
        for (; ub < units; ub += per) {
            const int u = ub + lane;
            uint32_t rm = 0, v0 = 0, r0 = 0;
            int x0 = 0, ry = 0, rz = 0;
            if (lane < per && u < units) {
                const int seg = u % nseg, row = u / nseg;
                x0 = lo[0] + 32 * seg;
                const int wd = min(32, hi[0] - x0);
                ry = lo[1] + row % ny;
                rz = lo[2] + row / ny;
                v0 = lin3(x0, ry, rz, sc);
                const uint32_t w0 = v0 >> 5, sh = v0 & 31u;
                uint64_t bits = __ldg(band.bits + w0);
                if (sh + (uint32_t)wd > 32u) bits |= (uint64_t)__ldg(band.bits + w0 + 1) << 32;
                rm = (uint32_t)(bits >> sh) & (wd >= 32 ? 0xffffffffu : ((1u << wd) - 1u));
                // band rank of v0 (whether or not v0 is in the band); bit b of
                // rm is vertex v0 + b, so its rank adds the set bits below b
                r0 = __ldg(band.prefix + w0) + __popc((uint32_t)bits & ((1u << sh) - 1u));
            }
            const uint32_t n = __popc(rm);
            uint32_t x = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            const uint32_t tot = __shfl_sync(0xffffffffu, x, 31);
            // (tot <= kPassVerts by the choice of `per`: an empty pass always takes the step)
            if (count > 0 && count + tot > (uint32_t)kPassVerts) break;  // run the pass, then this step again
            uint32_t slot = count + x - n;
            for (uint32_t m = rm; m; m &= m - 1u) {
                const int bx = __ffs(m) - 1;
                vloc[slot] = vert_loc(x0 + bx - lo[0], ry - lo[1], rz - lo[2]);
                vrank[slot++] = r0 + __popc(rm & ((1u << bx) - 1u));
            }
            count += tot;
        }
        __syncwarp();
        if (count > 0) pass(count);
    }
}

// The unscaled kernel's part of the field at vertex v, sum_j c_j (1 - |x_j -
// v|^2)^3 over the group's non-involved candidates j, is one polynomial in
// v for the whole group when every candidate is inside the support of every
// vertex (then no term is cut at q2 = 1).  With y_j = x_j - o, z = v - o
// (o: the centre of the group's vertex box), a_j = 1 - |y_j|^2, w = |z|^2:
//   1 - |x_j - v|^2 = (a_j - w) + 2 y_j.z, and the cube of that sums to
//   sum c (a-w)^3 + 6 sum c (a-w)^2 (y.z) + 12 sum c (a-w) (y.z)^2 + 8 sum c (y.z)^3,
// which needs 35 moments of (c, a, y): A_k = sum c a^k (k = 0..3),
// B_k = sum c a^k y (k = 0..2), C_k = sum c a^k y y^T (k = 0, 1) and
// D = sum c y y y.  The expansion holds exactly; it is used when
// max |y| + max |z| < 0.5 (all pairs well inside the unit support, every
// term of order 1, no cancellation), else the candidates are streamed.

struct MomAcc {
    float m[kMoments];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int k = 0; k < kMoments; ++k) m[k] = 0.f;
    }
    __device__ __forceinline__ void add(float c, float yx, float yy, float yz)
    {
        const float a = 1.0f - fmaf(yx, yx, fmaf(yy, yy, yz * yz));
        const float ca = c * a, ca2 = ca * a;
        m[0] += c;
        m[1] += ca;
        m[2] += ca2;
        m[3] += ca2 * a;
        m[4] = fmaf(c, yx, m[4]);   m[5] = fmaf(c, yy, m[5]);   m[6] = fmaf(c, yz, m[6]);
        m[7] = fmaf(ca, yx, m[7]);  m[8] = fmaf(ca, yy, m[8]);  m[9] = fmaf(ca, yz, m[9]);
        m[10] = fmaf(ca2, yx, m[10]); m[11] = fmaf(ca2, yy, m[11]); m[12] = fmaf(ca2, yz, m[12]);
        const float cx = c * yx, cy = c * yy, cz = c * yz;
        m[13] = fmaf(cx, yx, m[13]); m[14] = fmaf(cy, yy, m[14]); m[15] = fmaf(cz, yz, m[15]);
        m[16] = fmaf(cx, yy, m[16]); m[17] = fmaf(cx, yz, m[17]); m[18] = fmaf(cy, yz, m[18]);
        m[19] = fmaf(cx * a, yx, m[19]); m[20] = fmaf(cy * a, yy, m[20]); m[21] = fmaf(cz * a, yz, m[21]);
        m[22] = fmaf(cx * a, yy, m[22]); m[23] = fmaf(cx * a, yz, m[23]); m[24] = fmaf(cy * a, yz, m[24]);
        const float cxx = cx * yx, cyy = cy * yy, czz = cz * yz;
        m[25] = fmaf(cxx, yx, m[25]);  // xxx
        m[26] = fmaf(cyy, yy, m[26]);  // yyy
        m[27] = fmaf(czz, yz, m[27]);  // zzz
        m[28] = fmaf(cxx, yy, m[28]);  // xxy
        m[29] = fmaf(cxx, yz, m[29]);  // xxz
        m[30] = fmaf(cyy, yx, m[30]);  // xyy
        m[31] = fmaf(cyy, yz, m[31]);  // yyz
        m[32] = fmaf(czz, yx, m[32]);  // xzz
        m[33] = fmaf(czz, yy, m[33]);  // yzz
        m[34] = fmaf(cx * yy, yz, m[34]);  // xyz
    }
};

// The polynomial at z = v - o.
__device__ __forceinline__ float unscaled_sum(const float* m, float zx, float zy, float zz)
{
    const float w = fmaf(zx, zx, fmaf(zy, zy, zz * zz));
    const float t1 = fmaf(w, fmaf(w, fmaf(-w, m[0], 3.0f * m[1]), -3.0f * m[2]), m[3]);
    const float b0 = fmaf(m[4], zx, fmaf(m[5], zy, m[6] * zz));
    const float b1 = fmaf(m[7], zx, fmaf(m[8], zy, m[9] * zz));
    const float b2 = fmaf(m[10], zx, fmaf(m[11], zy, m[12] * zz));
    const float t2 = 6.0f * fmaf(w, fmaf(w, b0, -2.0f * b1), b2);
    const float xx = zx * zx, yy = zy * zy, zz2 = zz * zz, xy = zx * zy, xz = zx * zz, yz = zy * zz;
    const float q0 = fmaf(m[13], xx, fmaf(m[14], yy, fmaf(m[15], zz2, 2.0f * fmaf(m[16], xy, fmaf(m[17], xz, m[18] * yz)))));
    const float q1 = fmaf(m[19], xx, fmaf(m[20], yy, fmaf(m[21], zz2, 2.0f * fmaf(m[22], xy, fmaf(m[23], xz, m[24] * yz)))));
    const float t3 = 12.0f * fmaf(-w, q0, q1);
    const float d3 = fmaf(m[25], xx * zx, fmaf(m[26], yy * zy, m[27] * zz2 * zz));
    const float d21 = fmaf(m[28], xx * zy, fmaf(m[29], xx * zz, fmaf(m[30], yy * zx,
                      fmaf(m[31], yy * zz, fmaf(m[32], zz2 * zx, m[33] * zz2 * zy)))));
    const float t4 = 8.0f * fmaf(6.0f, m[34] * xy * zz, fmaf(3.0f, d21, d3));
    return (t1 + t2) + (t3 + t4);
}

// One warp per window group, groups handed out dynamically; no block-wide
// barriers.  The warp walks the group's index box 32 vertices at a time and
// collects up to 256 band vertices per pass (8 tiles of 32).  Per pass it
// streams the window's candidates 32 at a time: each lane loads one
// candidate's record into the warp's shared-memory slice once (candidates
// that reach none of the pass's tiles are dropped first), then for every
// tile the warp keeps the candidates whose support sphere reaches the
// tile's box and each lane adds their terms for its vertex of that tile.
// A vertex's sum takes the candidates in window order.
__global__ void __launch_bounds__(kFT, FSR_FIELD_MIN_BLOCKS) k_field_aniso_grouped(GroupArgs a, uint32_t ratio, Counters* ctr)
{
    __shared__ WarpSlice slices[kFWarps];
    const int lane = threadIdx.x & 31;
    WarpSlice& w = slices[threadIdx.x >> 5];
    const uint32_t nb = min(ctr->n_band, a.cap);
    const uint32_t ngroups = ctr->n_groups;  // groups holding band vertices
    const uint32_t nslab = field_slabs(ngroups);

    for (;;) {
        uint32_t k = 0;
        if (lane == 0) k = atomicAdd(&ctr->work_field, 1u);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= ngroups * nslab) break;
        const uint32_t g = a.glist[k / nslab];
        int c[3], lo[3], hi[3];
        if (!group_box(g, a.sp, a.sc, ratio, c, lo, hi) || !slab_box(k % nslab, nslab, lo, hi)) continue;
        bool tables = false;
        uint32_t total = 0;

        auto pass = [&](uint32_t nv) {
            if (!tables) {
                const float b0[3] = {vpos1(lo[0], a.sc.min[0], a.sc.cs), vpos1(lo[1], a.sc.min[1], a.sc.cs),
                                     vpos1(lo[2], a.sc.min[2], a.sc.cs)};
                const float b1[3] = {vpos1(hi[0] - 1, a.sc.min[0], a.sc.cs), vpos1(hi[1] - 1, a.sc.min[1], a.sc.cs),
                                     vpos1(hi[2] - 1, a.sc.min[2], a.sc.cs)};
                total = warp_candidates(a.sp, a.ranges, a.invol, a.reach, c, b0, b1, w);
                tables = true;
                // moments of the non-involved candidates about the box centre
                const float ox = 0.5f * (b0[0] + b1[0]), oy = 0.5f * (b0[1] + b1[1]), oz = 0.5f * (b0[2] + b1[2]);
                const float hx = 0.5f * (b1[0] - b0[0]), hy = 0.5f * (b1[1] - b0[1]), hz = 0.5f * (b1[2] - b0[2]);
                MomAcc acc;
                acc.zero();
                float y2max = 0.f;
                const CandTables tabs{w.cstart, w.cpre, w.cinv};
                for (uint32_t j = w.total_inv + lane; j < total; j += 32) {
                    int cell;
                    const uint32_t i = candidate(j, tabs, &cell, (int)w.ncells);
                    const float4 sm = __ldg(&a.smoothed[i]);
                    const float yx = sm.x - ox, yy = sm.y - oy, yz = sm.z - oz;
                    y2max = fmaxf(y2max, fmaf(yx, yx, fmaf(yy, yy, yz * yz)));
                    acc.add(a.sigma * sm.w, yx, yy, yz);
                }
#pragma unroll
                for (int k = 0; k < kMoments; ++k) {
                    float v = acc.m[k];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0) w.mom[k] = v;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) y2max = fmaxf(y2max, __shfl_xor_sync(0xffffffffu, y2max, o));
                const float zmax = sqrtf(fmaf(hx, hx, fmaf(hy, hy, hz * hz)));
                if (lane == 0) w.use_mom = (sqrtf(y2max) + zmax) * 1.001f < 0.5f ? 1u : 0u;
                __syncwarp();
            }
            const uint32_t ntiles = (nv + 31) / 32;
            // the pass's box, brick order and tile boxes
            float4 pl, ph;
            pass_layout(w.vloc, lo, a.sc, w.order, reinterpret_cast<uint32_t*>(&w.psum[0][0]), w.box, nv,
                        1.0f / a.sc.cs, lane, pl, ph);  // psum is zeroed below
            // two sums per vertex: the involved particles' terms, then the
            // non-involved particles' (the unscaled kernel: about 1e-7 each,
            // thousands of them) and the rounding errors of the first sum,
            // added among themselves and joined at the end, so that FP32
            // rounding does not drop or inflate them against a sum of order 1
            // the sums live in the warp's shared slice, so that the tile loops
            // need not be unrolled (the kernel's code stays small enough for
            // the instruction cache)
            for (int t = 0; t < kPassTiles; ++t) w.psum[t][lane] = w.usum[t][lane] = 0.f;
            const uint32_t total_inv = w.total_inv;
            // involved candidates: staged with their G, culled per tile by
            // their support sphere, evaluated two at a time
            uint32_t k0 = 0;
            for (uint32_t cb = 0; cb < total_inv; cb += 32) {
                const uint32_t j = cb + lane;
                bool keep = false;
                float4 r0 = make_float4(0.f, 0.f, 0.f, -1.f);
                const int cell = chunk_cell(cb, lane, w.cpre, w.ncells, k0);
                if (j < total_inv) {
                    const uint32_t i = w.cstart[cell] + (j - w.cpre[cell]);
                    // the three loads in flight together (most candidates are kept)
                    const float4* qsrc = a.qrec + 3ull * i;
                    r0 = __ldg(qsrc);
                    const float4 r1 = __ldg(qsrc + 1), r2 = __ldg(qsrc + 2);
                    keep = reaches(r0, pl, ph);
                    if (keep) stage_record(reinterpret_cast<float2*>(w.rec), lane, r0, r1, r2);
                }
                const uint32_t any = __ballot_sync(0xffffffffu, keep);
                __syncwarp();
                if (any) {
#pragma unroll 1
                    for (int t = 0; t < kPassTiles; ++t) {
                        if ((uint32_t)t < ntiles) {
                            const uint32_t m = __ballot_sync(0xffffffffu, keep && reaches(r0, w.box[2 * t], w.box[2 * t + 1]));
                            if (m) {
                                // the candidates that reach the tile, listed in
                                // lane order two to a pair block
                                if ((m >> lane) & 1u)
                                    list_pair_record(reinterpret_cast<const float2*>(w.rec), lane,
                                                     reinterpret_cast<float*>(w.lst), __popc(m & ((1u << lane) - 1u)));
                                __syncwarp();
                                const uint32_t v = 32 * t + lane;
                                if (v < nv) {
                                    const float4 vp = vert_pos(w.vloc[w.order[v]], lo, a.sc);
                                    // the chunk's terms are summed on their own and
                                    // then added to the vertex's sum with the
                                    // rounding error of that addition (two-sum)
                                    // kept in the second sum: with tens of
                                    // thousands of neighbours one running FP32 sum
                                    // drifts by more than 1e-5 of the field
                                    float s = 0.f;
                                    // one pair block per step, both candidates
                                    // evaluated at once by packed operations; the
                                    // terms of vertices inside the support enter
                                    // the sum in list (lane) order
                                    const float2 nvx = make_float2(-vp.x, -vp.x), nvy = make_float2(-vp.y, -vp.y),
                                                 nvz = make_float2(-vp.z, -vp.z);
                                    const uint32_t cnt = __popc(m);
                                    // not unrolled: copies of the body crowd the
                                    // instruction cache (measured: fetch stalls
                                    // doubled and the 2^18-particle frame slowed)
#pragma unroll 1
                                    for (uint32_t j = 0; j < cnt; j += 2) {
                                        float2 q2, u3, c;
                                        pair_terms(w.lst + (j >> 1) * kPairF4, nvx, nvy, nvz, q2, u3, c);
                                        if (q2.x < 1.0f) s = fmaf(c.x, u3.x, s);
                                        if (j + 1 < cnt && q2.y < 1.0f) s = fmaf(c.y, u3.y, s);
                                    }
                                    const float a0 = w.psum[t][lane];
                                    const float t0 = a0 + s;
                                    const float bp = t0 - a0;
                                    w.psum[t][lane] = t0;
                                    w.usum[t][lane] += (a0 - (t0 - bp)) + (s - bp);
                                }
                                __syncwarp();
                            }
                        }
                    }
                }
                __syncwarp();
            }
            // non-involved candidates: G = I and support 1 (world units), which
            // reaches every vertex of the window.  Their sum is the group's
            // moment polynomial when it applies; else they are streamed: only
            // the position and the coefficient sigma m / rho are staged, and
            // q2 is |x~ - v|^2
            const bool use_mom = w.use_mom != 0u;
            if (use_mom) {
                const float ox = 0.5f * (vpos1(lo[0], a.sc.min[0], a.sc.cs) + vpos1(hi[0] - 1, a.sc.min[0], a.sc.cs));
                const float oy = 0.5f * (vpos1(lo[1], a.sc.min[1], a.sc.cs) + vpos1(hi[1] - 1, a.sc.min[1], a.sc.cs));
                const float oz = 0.5f * (vpos1(lo[2], a.sc.min[2], a.sc.cs) + vpos1(hi[2] - 1, a.sc.min[2], a.sc.cs));
#pragma unroll 1
                for (int t = 0; t < kPassTiles; ++t) {
                    const uint32_t v = 32 * t + lane;
                    if ((uint32_t)t < ntiles && v < nv) {
                        const float4 vp = vert_pos(w.vloc[w.order[v]], lo, a.sc);
                        w.usum[t][lane] += unscaled_sum(w.mom, vp.x - ox, vp.y - oy, vp.z - oz);
                    }
                }
            }
            k0 = w.ninv_cells;
            for (uint32_t cb = use_mom ? total : total_inv; cb < total; cb += 32) {
                const uint32_t j = cb + lane;
                const int cell = chunk_cell(cb, lane, w.cpre, w.ncells, k0);
                if (j < total) {
                    const uint32_t i = w.cstart[cell] + (j - w.cpre[cell]);
                    const float4 sm = __ldg(&a.smoothed[i]);
                    w.rec[lane] = make_float4(sm.x, sm.y, sm.z, a.sigma * sm.w);
                }
                const uint32_t cnt = min(32u, total - cb);
                __syncwarp();
#pragma unroll 1
                for (int t = 0; t < kPassTiles; ++t) {
                    const uint32_t v = 32 * t + lane;
                    if ((uint32_t)t < ntiles && v < nv) {
                        const float4 vp = vert_pos(w.vloc[w.order[v]], lo, a.sc);
                        float su = 0.f;  // the chunk's terms, as for the involved candidates
                        uint32_t k = 0;
                        for (; k + 2 <= cnt; k += 2) {
                            const float4 qa = w.rec[k], qb = w.rec[k + 1];
                            const float ax = qa.x - vp.x, ay = qa.y - vp.y, az = qa.z - vp.z;
                            const float bx = qb.x - vp.x, by = qb.y - vp.y, bz = qb.z - vp.z;
                            const float q2a = fmaf(ax, ax, fmaf(ay, ay, az * az));
                            const float q2b = fmaf(bx, bx, fmaf(by, by, bz * bz));
                            const float ua = 1.0f - q2a, ub = 1.0f - q2b;
                            if (q2a < 1.0f) su = fmaf(qa.w, ua * ua * ua, su);
                            if (q2b < 1.0f) su = fmaf(qb.w, ub * ub * ub, su);
                        }
                        if (k < cnt) {
                            const float4 qa = w.rec[k];
                            const float ax = qa.x - vp.x, ay = qa.y - vp.y, az = qa.z - vp.z;
                            const float q2a = fmaf(ax, ax, fmaf(ay, ay, az * az));
                            const float ua = 1.0f - q2a;
                            if (q2a < 1.0f) su = fmaf(qa.w, ua * ua * ua, su);
                        }
                        w.usum[t][lane] += su;
                    }
                }
                __syncwarp();
            }
#pragma unroll
            for (int t = 0; t < kPassTiles; ++t) {
                const uint32_t v = 32 * t + lane;
                if (v < nv) {
                    const uint32_t rank = w.vrank[w.order[v]];
                    if (rank < nb) a.phi[rank] = (w.psum[t][lane] + w.usum[t][lane]) - 0.5f;
                }
            }
            __syncwarp();
        };

        list_band_vertices(a.sc, a.band, lo, hi, w.vloc, w.vrank, lane, pass);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- ZB05 / TC01
// updateScalarFieldValueZB05 (cu:230-289) and updateScalarFieldValueTC01
// (cu:178-227) grouped like the anisotropic field: a band vertex's
// candidates are the particles of the +-1 cells around its cell, the same for
// every vertex of the cell, so one warp streams them once per pass of up to
// 256 vertices and, per brick tile, evaluates only those within h of the
// tile's box.  Each vertex sums its terms in window order (cells z, y, x,
// particles in sorted order); candidates of the window cells the per-vertex
// walk narrows away lie beyond h and add nothing.
struct IsoSlice {
    float4 lst[32];                // one tile's candidates in lane order, two to a pair block (list_iso_pair)
    uint32_t vloc[kPassVerts];     // the pass's band vertices: index in the group's box (vert_loc)
    uint32_t vrank[kPassVerts];    // and band rank
    float4 box[2 * kPassTiles];    // per tile: lo, hi
    float sum[4][kPassTiles][32];  // per vertex: weight sum, then (ZB05) sum w (x - v)
    uint16_t order[kPassVerts];    // the pass's vertices in brick order
    uint32_t rb[9], rp[10];        // the window's rows: first particle, prefix of lengths
};

__device__ __forceinline__ bool within(float4 q, float4 lo, float4 hi, float r2)
{
    const float gx = fmaxf(0.f, fmaxf(lo.x - q.x, q.x - hi.x));
    const float gy = fmaxf(0.f, fmaxf(lo.y - q.y, q.y - hi.y));
    const float gz = fmaxf(0.f, fmaxf(lo.z - q.z, q.z - hi.z));
    return fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < r2;
}

// A tile's candidates listed two to a pair block of 2 float4: entry pos in
// the x and z components, entry pos + 1 in y and w,
//   (x, x') (y, y') | (z, z') (unused)
// so that the offsets and squared distances of both are formed by packed
// FP32x2 operations.
__device__ __forceinline__ void list_iso_pair(float4 q, float* lst, uint32_t pos)
{
    float* d = lst + (pos >> 1) * 8 + (pos & 1u);
    d[0] = q.x;
    d[2] = q.y;
    d[4] = q.z;
}

template <bool TC01>
__global__ void __launch_bounds__(kFT) k_field_iso_grouped(IsoFieldArgs a, BandView band, uint32_t ratio, Counters* ctr)
{
    __shared__ IsoSlice slices[kFWarps];
    const int lane = threadIdx.x & 31;
    IsoSlice& w = slices[threadIdx.x >> 5];
    const uint32_t nb = min(ctr->n_band, a.cap);
    const uint32_t ngroups = ctr->n_groups;  // groups holding band vertices
    const uint32_t nslab = field_slabs(ngroups);
    const float cr = cull_radius(a.h, a.sp.cs), cr2 = cr * cr;
    constexpr int kSums = TC01 ? 1 : 4;

    for (;;) {
        uint32_t k = 0;
        if (lane == 0) k = atomicAdd(&ctr->work_field, 1u);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= ngroups * nslab) break;
        const uint32_t g = a.glist[k / nslab];
        int c[3], lo[3], hi[3];
        if (!group_box(g, a.sp, a.sc, ratio, c, lo, hi) || !slab_box(k % nslab, nslab, lo, hi)) continue;
        // rows of the +-1 window (clamped as window() clamps), z then y
        if (lane < 9) {
            const int x0 = clampi(c[0] - 1, 0, (int)a.sp.res[0] - 1), x1 = clampi(c[0] + 1, 0, (int)a.sp.res[0] - 1);
            const int y0 = clampi(c[1] - 1, 0, (int)a.sp.res[1] - 1), y1 = clampi(c[1] + 1, 0, (int)a.sp.res[1] - 1);
            const int z0 = clampi(c[2] - 1, 0, (int)a.sp.res[2] - 1), z1 = clampi(c[2] + 1, 0, (int)a.sp.res[2] - 1);
            const int yy = y0 + lane % 3, zz = z0 + lane / 3;
            uint32_t beg = kEmpty, end = 0;
            if (yy <= y1 && zz <= z1) {
                const uint32_t c0 = lin3(x0, yy, zz, a.sp);
                for (int xx = 0; xx <= x1 - x0; ++xx) {
                    const uint2 r = __ldg(&a.ranges[c0 + xx]);
                    if (r.x != kEmpty) {
                        beg = min(beg, r.x);
                        end = max(end, r.y);
                    }
                }
            }
            w.rb[lane] = beg;
            w.rp[lane + 1] = beg == kEmpty ? 0u : end - beg;  // lengths for now
        }
        __syncwarp();
        if (lane == 0) {
            uint32_t acc = 0;
            for (int r = 0; r < 9; ++r) {
                const uint32_t len = w.rp[r + 1];
                w.rp[r] = acc;
                acc += len;
            }
            w.rp[9] = acc;
        }
        __syncwarp();
        const uint32_t total = w.rp[9];

        auto pass = [&](uint32_t nv) {
            float4 pl, ph;
            pass_layout(w.vloc, lo, a.sc, w.order, reinterpret_cast<uint32_t*>(&w.sum[0][0][0]), w.box, nv,
                        1.0f / a.sc.cs, lane, pl, ph);  // the sums are zeroed next
            const uint32_t ntiles = (nv + 31) / 32;
            for (int k = 0; k < kSums; ++k)
                for (int t = 0; t < kPassTiles; ++t) w.sum[k][t][lane] = 0.f;
            __syncwarp();
            for (uint32_t cb = 0; cb < total; cb += 32) {
                const uint32_t j = cb + lane;
                bool keep = false;
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                if (j < total) {
                    int r = 0;
                    while (r < 8 && w.rp[r + 1] <= j) ++r;
                    q = __ldg(&a.sorted[w.rb[r] + (j - w.rp[r])]);
                    keep = within(q, pl, ph, cr2);
                }
                const uint32_t any = __ballot_sync(0xffffffffu, keep);
                __syncwarp();
                if (any) {
#pragma unroll 1
                    for (int t = 0; t < kPassTiles; ++t) {
                        if ((uint32_t)t >= ntiles) break;
                        const uint32_t m = __ballot_sync(0xffffffffu, keep && within(q, w.box[2 * t], w.box[2 * t + 1], cr2));
                        if (!m) continue;
                        // the candidates within h of the tile, listed in lane
                        // order two to a pair block
                        if ((m >> lane) & 1u)
                            list_iso_pair(q, reinterpret_cast<float*>(w.lst), __popc(m & ((1u << lane) - 1u)));
                        __syncwarp();
                        const uint32_t v = 32 * t + lane;
                        if (v < nv) {
                            const float4 vp = vert_pos(w.vloc[w.order[v]], lo, a.sc);
                            float ws = w.sum[0][t][lane];
                            float ax = 0.f, ay = 0.f, az = 0.f;
                            if (!TC01) {
                                ax = w.sum[1][t][lane];
                                ay = w.sum[2][t][lane];
                                az = w.sum[3][t][lane];
                            }
                            const float2 nvx = make_float2(-vp.x, -vp.x), nvy = make_float2(-vp.y, -vp.y),
                                         nvz = make_float2(-vp.z, -vp.z);
                            const uint32_t cnt = __popc(m);
                            // one pair block per step: offsets and squared
                            // distances of both by packed operations (the
                            // roundings of the scalar forms), the rest per
                            // candidate; terms added in list (lane) order.  Not
                            // unrolled: copies of the body crowd the
                            // instruction cache
#pragma unroll 1
                            for (uint32_t j = 0; j < cnt; j += 2) {
                                const bool two = j + 1 < cnt;
                                const float4 A = w.lst[j], B = w.lst[j + 1];  // pair block j / 2
                                const float2 dx = __fadd2_rn(make_float2(A.x, A.y), nvx);
                                const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nvy);
                                const float2 dz = __fadd2_rn(make_float2(B.x, B.y), nvz);
                                const float2 d2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                                const float dxa = dx.x, dya = dy.x, dza = dz.x, d2a = d2.x;
                                const float dxb = dx.y, dyb = dy.y, dzb = dz.y, d2b = d2.y;
                                if (TC01) {
                                    const float ua = d2a * a.inv_h2 * 0.5f, ub = d2b * a.inv_h2 * 0.5f;
                                    const float ta = ua * ua - ua + 0.25f, tb = ub * ub - ub + 0.25f;
                                    if (d2a <= a.h2) ws += ta;
                                    if (two && d2b <= a.h2) ws += tb;
                                } else {
                                    const float ua = 1.0f - d2a * a.inv_h2, ub = 1.0f - d2b * a.inv_h2;
                                    const float wa = ua * ua * ua, wb = ub * ub * ub;
                                    if (d2a < a.h2) {
                                        ws += wa;
                                        ax = fmaf(dxa, wa, ax);
                                        ay = fmaf(dya, wa, ay);
                                        az = fmaf(dza, wa, az);
                                    }
                                    if (two && d2b < a.h2) {
                                        ws += wb;
                                        ax = fmaf(dxb, wb, ax);
                                        ay = fmaf(dyb, wb, ay);
                                        az = fmaf(dzb, wb, az);
                                    }
                                }
                            }
                            w.sum[0][t][lane] = ws;
                            if (!TC01) {
                                w.sum[1][t][lane] = ax;
                                w.sum[2][t][lane] = ay;
                                w.sum[3][t][lane] = az;
                            }
                        }
                        __syncwarp();  // the list is rewritten for the next tile
                    }
                }
                __syncwarp();
            }
            for (int t = 0; t < (int)ntiles; ++t) {
                const uint32_t v = 32 * t + lane;
                if (v < nv) {
                    const uint32_t rank = w.vrank[w.order[v]];
                    if (rank < nb) {
                        const float ws = w.sum[0][t][lane];
                        if (TC01) {
                            a.phi[rank] = ws;
                        } else {
                            const float ax = w.sum[1][t][lane], ay = w.sum[2][t][lane], az = w.sum[3][t][lane];
                            // |v - sum w p / sum w| = |sum w (p - v)| / sum w; a vertex with no
                            // weight keeps 0, the reference's memset value (cu:284)
                            a.phi[rank] = ws > 0.f ? sqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az))) / ws - a.rp : 0.f;
                            if (a.mv) {
                                const float inv = ws > 0.f ? 1.0f / ws : 0.f;
                                a.mv[rank] = make_float4(ax * inv, ay * inv, az * inv, ws);
                            }
                        }
                    }
                }
            }
            __syncwarp();
        };
        list_band_vertices(a.sc, band, lo, hi, w.vloc, w.vrank, lane, pass);
        __syncwarp();
    }
}

// The group box's vertices with a non-zero dL/dphi, listed in 4 x 4 x 2
// bricks of the box, so that each 32 consecutive ones (which share one
// culling box in the ZB05/TC01 adjoint) lie close together: a count per brick, a scan,
// then a scatter (the order inside a brick is that of the atomics; it changes
// no sum but the float atomics' order, which is not fixed anyway).
// emit(slot, lx, ly, lz, rank, gv) stores one vertex (slots below `cap` only);
// hist holds `cap` words.  Every thread of the block calls it; returns the
// number of such vertices.
template <class Emit>
__device__ uint32_t list_grad_vertices(const BandView& band, const float* __restrict__ gphi, uint32_t nb,
                                       const Grid& sc, const int lo[3], const int hi[3], uint32_t* hist, uint32_t cap,
                                       uint32_t* s_tot, Emit&& emit)
{
    const int tid = threadIdx.x, lane = tid & 31;
    const int nx = hi[0] - lo[0], ny = hi[1] - lo[1], nz = hi[2] - lo[2];
    const int nbox = nx * ny * nz;
    const int bx = (nx + 3) / 4, by = (ny + 3) / 4, bz = (nz + 1) / 2;
    const bool bricks = (uint32_t)(bx * by * bz) <= cap;  // (always, for boxes within the capacity)
    const int nbins = bricks ? bx * by * bz : 1;
    auto key = [&](int lx, int ly, int lz) { return bricks ? (lx >> 2) + bx * ((ly >> 2) + by * (lz >> 1)) : 0; };
    auto grad = [&](int i, int& lx, int& ly, int& lz, uint32_t& rank) -> float {
        lx = i % nx;
        ly = (i / nx) % ny;
        lz = i / (nx * ny);
        const uint32_t v = lin3(lo[0] + lx, lo[1] + ly, lo[2] + lz, sc);
        if (!band_has(band, v)) return 0.f;
        rank = band_rank(band, v);
        return rank < nb ? __ldg(gphi + rank) : 0.f;
    };
    for (int b = tid; b < nbins; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    for (int i = tid; i < nbox; i += blockDim.x) {
        int lx, ly, lz;
        uint32_t rank = 0;
        if (grad(i, lx, ly, lz, rank) != 0.f) atomicAdd(&hist[key(lx, ly, lz)], 1u);
    }
    __syncthreads();
    if (tid < 32) {  // exclusive scan of the counts
        uint32_t run = 0;
        for (int b0 = 0; b0 < nbins; b0 += 32) {
            const int b = b0 + lane;
            const uint32_t cnt = b < nbins ? hist[b] : 0u;
            uint32_t x = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (b < nbins) hist[b] = run + x - cnt;
            run += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) *s_tot = run;
    }
    __syncthreads();
    for (int i = tid; i < nbox; i += blockDim.x) {
        int lx, ly, lz;
        uint32_t rank = 0;
        const float gv = grad(i, lx, ly, lz, rank);
        if (gv != 0.f) {
            const uint32_t slot = atomicAdd(&hist[key(lx, ly, lz)], 1u);
            if (slot < cap) emit(slot, lx, ly, lz, rank, gv);
        }
    }
    __syncthreads();
    return *s_tot;
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
    const float4* qrec;
    const float4* smoothed;
    const uint2* ranges;
    const uint8_t* invol;
    const float* reach;
    const float* gphi;
    uint32_t* glist;
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
    __shared__ uint32_t s_nv, s_tot, s_wsum[4], s_next;
    __shared__ float4 s_lo, s_hi;
    const CandTables tabs{cstart, cpre, cinv};

    __shared__ uint32_t s_g;
    const uint32_t nb = min(ctr->n_band, a.cap);
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t nlist = a.glist[0];

    // the groups holding gradient vertices, handed out one per block from
    // the list k_mark_keys built
    for (;;) {
        if (tid == 0) s_g = atomicAdd(&a.glist[1], 1u);
        __syncthreads();
        const uint32_t k = s_g;
        __syncthreads();
        if (k >= nlist) break;
        const uint32_t g = a.glist[4 + k];
        int c[3], lo[3], hi[3];
        if (!group_box(g, a.sp, a.sc, ratio, c, lo, hi)) continue;
        const int nx = hi[0] - lo[0], ny = hi[1] - lo[1], nz = hi[2] - lo[2];
        const int nbox = nx * ny * nz;

        // 1. the group's vertices with dL/dphi != 0 (listed in scan order:
        // brick order, as in the ZB05 adjoint, measured slower here)
        if (tid == 0) {
            s_nv = 0;
            s_next = 0;
        }
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

        // 3. one candidate per thread, gradient kept in registers; warps take
        // the next 32 candidates as they finish, so that the group's slow
        // candidates do not hold the others at the block's barrier
        for (;;) {
            uint32_t cb = 0;
            if (lane == 0) cb = atomicAdd(&s_next, 32u);
            cb = __shfl_sync(0xffffffffu, cb, 0);
            if (cb >= total) break;
            const uint32_t j = cb + lane;
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
            if (!inv) {
                // unscaled kernel (G = I, support 1): d/dx~ (1 - |r|^2)^3 = -6 (1 - |r|^2)^2 r;
                // no dL/dG.  Candidates come cell by cell, so a warp's threads
                // mostly take the same branch.
                for (uint32_t q = 0; q < nv; ++q) {
                    const float4 v = av[q];
                    const float rx = r0.x - v.x, ry = r0.y - v.y, rz = r0.z - v.z;
                    const float q2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                    if (!(q2 < 1.0f)) continue;
                    const float u = 1.0f - q2;
                    const float A = -6.0f * v.w * coef * u * u;
                    gxs = fmaf(A, rx, gxs);
                    gys = fmaf(A, ry, gys);
                    gzs = fmaf(A, rz, gzs);
                }
                if (gxs != 0.f || gys != 0.f || gzs != 0.f) atomicAdd(a.gsmooth + i, make_float4(gxs, gys, gzs, 0.f));
                continue;
            }
            // per pair, with M = G^T G (the forward's quadratic form) and
            // B = -3 g c (1 - q2)^2:  dL/dx~ += 2 B M d,  dL/dM += B d d^T
            // (S, symmetric); dL/dG = 2 G S once per candidate at the end
            const float4 qa = __ldg(a.qrec + 3ull * i + 1), qb = __ldg(a.qrec + 3ull * i + 2);
            const float m00 = qa.x, m01 = 0.5f * qa.y, m02 = 0.5f * qa.z;
            const float m11 = qb.x, m12 = 0.5f * qb.y, m22 = qb.z;
            float s00 = 0.f, s01 = 0.f, s02 = 0.f, s11 = 0.f, s12 = 0.f, s22 = 0.f;
            for (uint32_t k = 0; k < nch; ++k) {
                if (!(box_dist2(r0.x, r0.y, r0.z, cbox[2 * k], cbox[2 * k + 1]) < r0.w)) continue;
                const uint32_t qe = min(nv, 32 * k + 32);
                for (uint32_t q = 32 * k; q < qe; ++q) {
                    const float4 v = av[q];
                    const float rx = r0.x - v.x, ry = r0.y - v.y, rz = r0.z - v.z;
                    const float d2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
                    if (!(d2 < r0.w)) continue;
                    const float a0 = fmaf(m00, rx, fmaf(m01, ry, m02 * rz));
                    const float a1 = fmaf(m01, rx, fmaf(m11, ry, m12 * rz));
                    const float a2 = fmaf(m02, rx, fmaf(m12, ry, m22 * rz));
                    const float q2 = fmaf(rx, a0, fmaf(ry, a1, rz * a2));
                    if (!(q2 < 1.0f)) continue;
                    const float u = 1.0f - q2;
                    const float B = -3.0f * v.w * coef * u * u;
                    const float B2 = B + B;
                    gxs = fmaf(B2, a0, gxs);
                    gys = fmaf(B2, a1, gys);
                    gzs = fmaf(B2, a2, gzs);
                    const float bx = B * rx, by = B * ry, bz = B * rz;
                    s00 = fmaf(bx, rx, s00);
                    s01 = fmaf(bx, ry, s01);
                    s02 = fmaf(bx, rz, s02);
                    s11 = fmaf(by, ry, s11);
                    s12 = fmaf(by, rz, s12);
                    s22 = fmaf(bz, rz, s22);
                    sc = fmaf(v.w, u * u * u, sc);
                }
            }
            if (gxs != 0.f || gys != 0.f || gzs != 0.f || sc != 0.f) {
                atomicAdd(a.gsmooth + i, make_float4(gxs, gys, gzs, sc));
                // dL/dG = 2 G S
                auto row = [&](float4 g) {
                    return make_float4(2.0f * (g.x * s00 + g.y * s01 + g.z * s02),
                                       2.0f * (g.x * s01 + g.y * s11 + g.z * s12),
                                       2.0f * (g.x * s02 + g.y * s12 + g.z * s22), 0.f);
                };
                atomicAdd(a.gG + 3ull * i, row(g0));
                atomicAdd(a.gG + 3ull * i + 1, row(g1));
                atomicAdd(a.gG + 3ull * i + 2, row(g2));
            }
        }
        __syncthreads();
    }
}

// Adjoint of the ZB05 / TC01 fields (updateScalarFieldValueZB05 cu:230-289,
// TC01 cu:178-227), grouped like the anisotropic adjoint: a group's vertices
// with dL/dphi != 0 (and, for ZB05, their (mean - v, weight sum) from the
// forward) sit in shared memory with one box per 32; the candidates are the
// particles of the +-1 cell window around the group's cell (the forward's
// window for each of those vertices), one per thread, and each adds its
// dL/dx over the active vertices within h with one float4 atomic.
template <bool TC01>
__global__ void __launch_bounds__(kBT) k_field_iso_backward_grouped(BwdArgs a, uint32_t vlist_cap, const Counters* ctr)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float4* av = reinterpret_cast<float4*>(smem);  // active vertices: (v, dL/dphi)
    // ZB05, per active vertex: e = (mean - v) dL/dphi / (|mean - v| W) and e.(mean - v), so that a pair
    // needs no square root or division (W: the weight sum; vertices without weight get 0)
    float4* am = av + vlist_cap;
    float4* cbox = am + (TC01 ? 0 : vlist_cap);     // per 32 of them: lo, hi
    uint32_t* hist = reinterpret_cast<uint32_t*>(cbox + 2 * ((vlist_cap + 31) / 32));  // vlist_cap words
    __shared__ uint32_t s_nv, s_rb[9], s_re[9], s_rp[10], s_next;
    const uint32_t nb = min(ctr->n_band, a.cap_band);
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t ngroups = (a.sp.res[0] + 1) * (a.sp.res[1] + 1) * (a.sp.res[2] + 1);
    const float h2 = a.h * a.h, inv_h2 = 1.0f / h2;
    const float cr = cull_radius(a.h, a.sp.cs), cr2 = cr * cr;
    __shared__ uint32_t s_g;
    const uint32_t nlist = a.glist[0];

    // the groups holding gradient vertices, handed out one per block from
    // the list k_mark_keys built
    for (;;) {
        if (tid == 0) s_g = atomicAdd(&a.glist[2], 1u);
        __syncthreads();
        const uint32_t k = s_g;
        __syncthreads();
        if (k >= nlist) break;
        const uint32_t g = a.glist[4 + k];
        int c[3], lo[3], hi[3];
        if (!group_box(g, a.sp, a.sc, a.ratio, c, lo, hi)) continue;
        if (tid == 0) s_next = 0;
        list_grad_vertices(a.band, a.gphi, nb, a.sc, lo, hi, hist, vlist_cap, &s_nv,
                           [&](uint32_t slot, int lx, int ly, int lz, uint32_t rank, float gv) {
            av[slot] = make_float4(vpos1(lo[0] + lx, a.sc.min[0], a.sc.cs), vpos1(lo[1] + ly, a.sc.min[1], a.sc.cs),
                                   vpos1(lo[2] + lz, a.sc.min[2], a.sc.cs), gv);
            if (!TC01) {
                const float4 m = __ldg(a.mv + rank);  // mean - v, weight sum
                const float ml = sqrtf(fmaf(m.x, m.x, fmaf(m.y, m.y, m.z * m.z)));
                float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
                if (m.w > 0.f && ml > 0.f) {
                    const float f = gv / ml / m.w;
                    e = make_float4(m.x * f, m.y * f, m.z * f, 0.f);
                    e.w = fmaf(e.x, m.x, fmaf(e.y, m.y, e.z * m.z));
                }
                am[slot] = e;
            }
        });
        // the +-1 window's rows (x-adjacent cells are contiguous in the sorted order)
        if (tid < 9) {
            const int x0 = clampi(c[0] - 1, 0, (int)a.sp.res[0] - 1), x1 = clampi(c[0] + 1, 0, (int)a.sp.res[0] - 1);
            const int y0 = clampi(c[1] - 1, 0, (int)a.sp.res[1] - 1), y1 = clampi(c[1] + 1, 0, (int)a.sp.res[1] - 1);
            const int z0 = clampi(c[2] - 1, 0, (int)a.sp.res[2] - 1), z1 = clampi(c[2] + 1, 0, (int)a.sp.res[2] - 1);
            const int yy = y0 + tid % 3, zz = z0 + tid / 3;
            uint32_t beg = kEmpty, end = 0;
            if (yy <= y1 && zz <= z1) {
                const uint32_t c0 = lin3(x0, yy, zz, a.sp);
                for (int xx = 0; xx <= x1 - x0; ++xx) {
                    const uint2 r = __ldg(&a.ranges[c0 + xx]);
                    if (r.x != kEmpty) {
                        beg = min(beg, r.x);
                        end = max(end, r.y);
                    }
                }
            }
            s_rb[tid] = beg;
            s_re[tid] = end > beg ? end : beg;
        }
        __syncthreads();
        const uint32_t nv = min(s_nv, vlist_cap);
        if (tid == 0) {
            uint32_t acc = 0;
            for (int r = 0; r < 9; ++r) {
                s_rp[r] = acc;
                acc += (s_rb[r] == kEmpty) ? 0u : s_re[r] - s_rb[r];
            }
            s_rp[9] = acc;
        }
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
        const uint32_t total = nv ? s_rp[9] : 0u;
        // one candidate per thread; warps take the next 32 as they finish
        for (;;) {
            uint32_t cb = 0;
            if (lane == 0) cb = atomicAdd(&s_next, 32u);
            cb = __shfl_sync(0xffffffffu, cb, 0);
            if (cb >= total) break;
            const uint32_t jj = cb + lane;
            if (jj >= total) continue;
            int r = 0;
            while (r < 8 && s_rp[r + 1] <= jj) ++r;
            const uint32_t j = s_rb[r] + (jj - s_rp[r]);
            const float4 q = __ldg(&a.sorted[j]);
            float gx = 0.f, gy = 0.f, gz = 0.f;
            for (uint32_t k = 0; k < nch; ++k) {
                if (!(box_dist2(q.x, q.y, q.z, cbox[2 * k], cbox[2 * k + 1]) < cr2)) continue;
                const uint32_t qe = min(nv, 32 * k + 32);
                for (uint32_t t = 32 * k; t < qe; ++t) {
                    const float4 v = av[t];
                    const float dx = q.x - v.x, dy = q.y - v.y, dz = q.z - v.z;
                    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    if (TC01) {
                        if (d2 > h2) continue;
                        const float tt = d2 * inv_h2 * 0.5f;
                        const float sg = v.w * (2.f * tt - 1.f) * inv_h2;
                        gx = fmaf(sg, dx, gx);
                        gy = fmaf(sg, dy, gy);
                        gz = fmaf(sg, dz, gz);
                    } else {
                        if (d2 >= h2) continue;
                        const float4 e = am[t];
                        const float u = 1.0f - d2 * inv_h2;
                        const float wt = u * u * u;
                        // d phi / d xbar = (xbar - v) / |xbar - v|; d xbar / d x_j = (w I + (x_j - xbar)
                        // (dw/dx_j)^T) / W with dw/dx_j = -6 u^2 (x_j - v) / h^2; with e as above
                        // (x_j - xbar = d - (mean - v)):
                        //   dL/dx_j += wt e + (e.d - e.(mean - v)) (-6 u^2 / h^2) d
                        const float k2 = (fmaf(e.x, dx, fmaf(e.y, dy, e.z * dz)) - e.w) * (-6.0f * u * u * inv_h2);
                        gx = fmaf(wt, e.x, fmaf(k2, dx, gx));
                        gy = fmaf(wt, e.y, fmaf(k2, dy, gy));
                        gz = fmaf(wt, e.z, fmaf(k2, dz, gz));
                    }
                }
            }
            if (gx != 0.f || gy != 0.f || gz != 0.f) atomicAdd(a.gx + j, make_float4(gx, gy, gz, 0.f));
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
    a.qrec = f.qrec;
    a.smoothed = f.smoothed;
    a.ranges = f.ranges;
    a.invol = f.invol;
    a.reach = f.cell_rmax;
    a.gphi = f.gphi;
    a.glist = f.glist;
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

void launch_field_aniso_grouped(const KernelCtx& c, const AnisoFieldArgs& f, const BandView& band, uint32_t ratio,
                                Counters* ctr)
{
    GroupArgs a;
    a.sp = f.sp;
    a.sc = f.sc;
    a.band = band;
    a.grec = f.grec;
    a.qrec = f.qrec;
    a.smoothed = f.smoothed;
    a.glist = f.glist;
    a.ranges = f.ranges;
    a.invol = f.invol;
    a.reach = f.cell_rmax;
    a.phi = f.phi;
    a.sigma = f.sigma;
    a.cap = f.cap;
    a.vlist_cap = 0;
    const uint64_t groups = (uint64_t)(f.sp.res[0] + 1) * (f.sp.res[1] + 1) * (f.sp.res[2] + 1);
    const unsigned grid = (unsigned)std::min<uint64_t>(
        (groups + kFWarps - 1) / kFWarps, std::max<uint64_t>(1, (uint64_t)c.num_sms * 16 / std::max(1, c.grid_div)));
    k_field_aniso_grouped<<<grid, kFT, 0, c.stream>>>(a, ratio, ctr);
    ++g_launches;
}

bool launch_field_iso_backward_grouped(const KernelCtx& c, const BwdArgs& a, bool tc01, const Counters* ctr)
{
    const uint32_t vcap = (a.ratio + 2) * (a.ratio + 2) * (a.ratio + 2);
    const size_t smem = sizeof(float4) * vcap * (tc01 ? 1 : 2) + sizeof(float4) * 2 * ((vcap + 31) / 32) +
                        sizeof(uint32_t) * vcap;
    if (smem > 200 * 1024) return false;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_field_iso_backward_grouped<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_field_iso_backward_grouped<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        configured = true;
    }
    const uint64_t groups = (uint64_t)(a.sp.res[0] + 1) * (a.sp.res[1] + 1) * (a.sp.res[2] + 1);
    const unsigned grid = (unsigned)std::min<uint64_t>(
        groups, std::max<uint64_t>(1, (uint64_t)c.num_sms * 8 / std::max(1, c.grid_div)));
    if (tc01) k_field_iso_backward_grouped<true><<<grid, kBT, smem, c.stream>>>(a, vcap, ctr);
    else k_field_iso_backward_grouped<false><<<grid, kBT, smem, c.stream>>>(a, vcap, ctr);
    ++g_launches;
    return true;
}

void launch_field_iso_grouped(const KernelCtx& c, bool tc01, const IsoFieldArgs& f, const BandView& band, uint32_t ratio,
                              Counters* ctr)
{
    const uint64_t groups = (uint64_t)(f.sp.res[0] + 1) * (f.sp.res[1] + 1) * (f.sp.res[2] + 1);
    const unsigned grid = (unsigned)std::min<uint64_t>(
        (groups + kFWarps - 1) / kFWarps, std::max<uint64_t>(1, (uint64_t)c.num_sms * 16 / std::max(1, c.grid_div)));
    if (tc01) k_field_iso_grouped<true><<<grid, kFT, 0, c.stream>>>(f, band, ratio, ctr);
    else k_field_iso_grouped<false><<<grid, kFT, 0, c.stream>>>(f, band, ratio, ctr);
    ++g_launches;
}

}  // namespace fsr
