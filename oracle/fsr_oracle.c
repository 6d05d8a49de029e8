/*
 * CPU oracle for the particle -> narrow band -> marching-cubes path.
 * TEST INFRASTRUCTURE ONLY: tests, the smoke check and the benchmark's CPU
 * baseline load it as the checker; the product never links or calls it.
 *
 * A restatement, stage by stage, of the reference pipeline
 * (FluidSurfaceReconstruction/GPU/ReconstructionCUDA.cu, "cu" below, and
 * ReconstructionCUDA.cuh, "cuh") on the reference's dense layouts; the
 * stage signatures are declared in fsr_stage_api.h.
 *
 * Two builds (see build_oracle.sh):
 *  - FSR_REAL_BITS=32: every floating-point operation is the reference's own
 *    FP32 (or, where the source promotes, FP64) operation in source order,
 *    evaluated without contraction (-ffp-contract=off).  The one substitute
 *    is the 3x3 SVD (GPU/SVD3.cuh, McAdams et al. 2011): the covariance is
 *    symmetric positive definite, so its SVD is its eigen-decomposition,
 *    computed here by cyclic Jacobi in FP64 and rounded to FP32 where the
 *    reference's SVD would return its factors.
 *  - FSR_REAL_BITS=64: the same algorithm with every continuous quantity
 *    (field sums, smoothed and mean positions, covariances, G, interpolated
 *    vertices and normals) carried in FP64.  Decisions the reference defines
 *    in FP32 - cell indices, grid vertex positions, band membership, surface
 *    flags and the neighbour counts of the covariance stage - keep their FP32
 *    definition so that both builds walk the same particles.
 *
 * Parity hazards reproduced on purpose (reference behaviour, not bugs here):
 * truncating cell index (cuh:354-358), surface test skipping the last cell
 * layer (cu:81), band extent fixed at 3 with an exclusive x bound (cu:569,
 * 582) and a double-precision radius test (cu:587), unscaled kernel for
 * non-involved particles (cu:888-899, cuh:312-322), ZB05 vertices with no
 * weight keeping the pre-filled value (cu:284).  Particles outside the grid
 * are rejected with an error here (the reference writes out of bounds,
 * cu:1391-1395).  The host marching cubes' out-of-grid reads
 * (MarchingCubesCPU.h:142-149) are defined as 0 here.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fsr_stage_api.h"
#include "fsr_mc_tables.h"

#ifndef FSR_REAL_BITS
#define FSR_REAL_BITS 32
#endif
#if FSR_REAL_BITS == 64
typedef double real_t;
#else
typedef float real_t;
#endif

#define EMPTY_CELL 0xFFFFFFFFu
#define OK 0
#define ERR_ARG (-1)
#define ERR_RANGE (-3)

/* SIGMA and EPSILON_ of cu:25-26. */
#if FSR_REAL_BITS == 32
static const float SIGMA_F = 315.0f / (64.0f * 3.1415926535898f);
#endif
static const float EPS_F = (float)1.0e-7;

/* ------------------------------------------------------------------ */
/* index helpers (cuh:338-358, 366-370, 402-416)                       */

typedef struct { int x, y, z; } i3;
typedef struct { float x, y, z; } f3;

static inline uint32_t lin3(uint32_t x, uint32_t y, uint32_t z, const uint32_t r[3])
{
    return z * r[0] * r[1] + y * r[0] + x; /* index3DTo1D, u32 arithmetic */
}

static inline void unlin3(uint32_t i, const uint32_t r[3], uint32_t* x, uint32_t* y, uint32_t* z)
{
    uint32_t xy = r[0] * r[1];
    *z = i / xy;
    uint32_t m = i % xy;
    *y = m / r[0];
    *x = m % r[0];
}

/* getIndex3D: truncation of (p - min) / cellSize, component-wise FP32 */
static inline i3 cell_of(f3 p, const o_gridinfo* g)
{
    i3 c;
    c.x = (int)((p.x - g->minPos[0]) / g->cellSize);
    c.y = (int)((p.y - g->minPos[1]) / g->cellSize);
    c.z = (int)((p.z - g->minPos[2]) / g->cellSize);
    return c;
}

/* getVertexPos: float(index) * cellSize + min, product rounded first */
static inline f3 vertex_pos(uint32_t x, uint32_t y, uint32_t z, const o_gridinfo* g)
{
    f3 v;
    v.x = (float)x * g->cellSize + g->minPos[0];
    v.y = (float)y * g->cellSize + g->minPos[1];
    v.z = (float)z * g->cellSize + g->minPos[2];
    return v;
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static inline f3 ld3(const float* p, uint32_t i)
{
    f3 r = {p[3 * (size_t)i], p[3 * (size_t)i + 1], p[3 * (size_t)i + 2]};
    return r;
}

/* window of cells c +- ext clamped to the grid (cu:194-199 and siblings) */
static inline void window(i3 c, int ext, const uint32_t r[3], i3* lo, i3* hi)
{
    lo->x = clampi(c.x - ext, 0, (int)r[0] - 1);
    lo->y = clampi(c.y - ext, 0, (int)r[1] - 1);
    lo->z = clampi(c.z - ext, 0, (int)r[2] - 1);
    hi->x = clampi(c.x + ext, 0, (int)r[0] - 1);
    hi->y = clampi(c.y + ext, 0, (int)r[1] - 1);
    hi->z = clampi(c.z + ext, 0, (int)r[2] - 1);
}

static inline uint64_t cells_of(const o_gridinfo* g)
{
    return (uint64_t)g->res[0] * g->res[1] * g->res[2];
}

int o_real_bytes(void) { return (int)sizeof(real_t); }

/* The marching-cubes tables in the reference's layout (MarchingCubesHelper.cpp:
 * 3-577): edge flags per case, triangle edge lists of 16 ints per case (-1
 * terminated), vertex counts per case, and the two corners of each edge.
 * For uploading to the reference's own kernels (oracle/ref_gpu). */
void o_mc_reference_tables(uint32_t edge_flags[256], int32_t tri[256 * 16], uint32_t nverts[256],
                           uint32_t edge_corners[24])
{
    for (unsigned c = 0; c < 256; ++c) {
        edge_flags[c] = fsr_o_edge_flags(c);
        nverts[c] = fsr_o_num_vertices(c);
        for (unsigned k = 0; k < 16; ++k) tri[16 * c + k] = k < 15 ? fsr_o_tri_edge(c, k) : -1;
    }
    for (unsigned e = 0; e < 12; ++e) {
        edge_corners[2 * e] = (uint32_t)FSR_O_EDGE[e][0];
        edge_corners[2 * e + 1] = (uint32_t)FSR_O_EDGE[e][1];
    }
}
int o_is_reference(void) { return 0; }
int o_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* grid derivation (ReconstructorGPU.cpp:237-268 spatial, :99-105 scalar)*/

int o_grid_derive(const float bbmin[3], const float bbmax[3], float h, float cellScale,
                  uint32_t ratio, o_gridinfo* sp, o_gridinfo* sc)
{
    if (!(h > 0.0f) || !(cellScale > 0.0f) || ratio == 0) return ERR_ARG;
    float cs = h * cellScale;
    for (int a = 0; a < 3; ++a) {
        sp->minPos[a] = bbmin[a] - cs;
        sp->maxPos[a] = bbmax[a] + cs;
    }
    sp->cellSize = cs;
    float scs = cs / (float)ratio;
    sc->cellSize = scs;
    for (int a = 0; a < 3; ++a) {
        sc->minPos[a] = sp->minPos[a];
        sc->maxPos[a] = sp->maxPos[a];
        float rs = (sp->maxPos[a] - sp->minPos[a]) / cs + 1.0f;
        float rv = (sc->maxPos[a] - sc->minPos[a]) / scs + 1.0f;
        if (!(rs >= 1.0f && rs < 4294967296.0f) || !(rv >= 1.0f && rv < 4294967296.0f)) return ERR_ARG;
        sp->res[a] = (uint32_t)rs;
        sc->res[a] = (uint32_t)rv;
    }
    return OK;
}

/* ------------------------------------------------------------------ */
/* spatial hashing: calcParticlesHashKernel (cu:1379-1396)               */

int o_hash(const float* pos, uint32_t n, const o_gridinfo* sp, uint32_t* keys, float* flag)
{
    int bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        f3 p = ld3(pos, (uint32_t)i);
        float q[3] = {(p.x - sp->minPos[0]) / sp->cellSize, (p.y - sp->minPos[1]) / sp->cellSize,
                      (p.z - sp->minPos[2]) / sp->cellSize};
        int ok = 1;
        for (int a = 0; a < 3; ++a)
            if (!(q[a] > -1.0f && q[a] < (float)sp->res[a])) ok = 0;
        if (!ok) { bad |= 1; keys[i] = EMPTY_CELL; continue; }
        i3 c = cell_of(p, sp);
        uint32_t k = lin3((uint32_t)c.x, (uint32_t)c.y, (uint32_t)c.z, sp->res);
        keys[i] = k;
#pragma omp atomic write
        flag[k] = 1.0f;
    }
    return bad ? ERR_RANGE : OK;
}

/* ------------------------------------------------------------------ */
/* surface cells and particles (cu:70-120, 466-551)                      */

static int surface_cell(uint32_t t, const float* flag, const o_gridinfo* sp)
{
    const uint32_t* r = sp->res;
    uint32_t x, y, z;
    unlin3(t, r, &x, &y, &z);
    if (x >= r[0] - 1 || y >= r[1] - 1 || z >= r[2] - 1) return 0; /* last layer skipped */
    if (flag[t] < 1.0f) return 0;
    i3 c = {(int)x, (int)y, (int)z}, lo, hi;
    window(c, 1, r, &lo, &hi);
    for (int zz = lo.z; zz <= hi.z; ++zz)
        for (int yy = lo.y; yy <= hi.y; ++yy)
            for (int xx = lo.x; xx <= hi.x; ++xx)
                if (flag[lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, r)] < 1.0f) return 1;
    return 0;
}

int o_surface(const o_simparam* p, const float* flag, const uint32_t* ranges,
              const o_gridinfo* sp, uint32_t* sflag, uint32_t n)
{
    (void)p; (void)n;
    const int64_t C = (int64_t)cells_of(sp);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t t = 0; t < C; ++t) {
        if (!surface_cell((uint32_t)t, flag, sp)) continue;
        uint32_t s = ranges[2 * t], e = ranges[2 * t + 1];
        if (s == EMPTY_CELL) continue;
        for (uint32_t i = s; i < e; ++i) sflag[i] = 1;
    }
    return OK;
}

int o_surface_involve(const o_simparam* p, const float* flag, const uint32_t* ranges,
                      const o_gridinfo* sp, uint32_t* sflag, uint32_t n, uint32_t* ninv)
{
    (void)p; (void)n;
    const uint32_t* r = sp->res;
    const int64_t C = (int64_t)cells_of(sp);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t t = 0; t < C; ++t) {
        if (!surface_cell((uint32_t)t, flag, sp)) continue;
        uint32_t s = ranges[2 * t], e = ranges[2 * t + 1];
        if (s != EMPTY_CELL)
            for (uint32_t i = s; i < e; ++i) sflag[i] = 1;
        uint32_t x, y, z;
        unlin3((uint32_t)t, r, &x, &y, &z);
        i3 c = {(int)x, (int)y, (int)z}, lo, hi;
        window(c, 2, r, &lo, &hi);
        for (int zz = lo.z; zz <= hi.z; ++zz)
            for (int yy = lo.y; yy <= hi.y; ++yy)
                for (int xx = lo.x; xx <= hi.x; ++xx) {
                    uint32_t k = lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, r);
                    if (ranges[2 * k] == EMPTY_CELL) continue;
                    uint32_t cnt = ranges[2 * k + 1] - ranges[2 * k];
#pragma omp atomic write
                    ninv[k] = cnt;
                }
    }
    return OK;
}

/* ------------------------------------------------------------------ */
/* narrow band: estimationOfSurfaceVertices (cu:554-595)                 */

int o_band(const o_simparam* p, const o_gridinfo* sc, const float* pos, const uint32_t* sflag,
           uint32_t n, const uint32_t* ranges, const o_gridinfo* sp, uint32_t* isSurf)
{
    (void)ranges; (void)sp;
    const uint32_t* r = sc->res;
    const double rad = (double)p->smoothingRadius * 1.5; /* double compare, cu:587 */
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)n; ++t) {
        if (sflag[t] == 0) continue;
        f3 q = ld3(pos, (uint32_t)t);
        i3 c = cell_of(q, sc), lo, hi;
        window(c, 3, r, &lo, &hi);
        for (int z = lo.z; z <= hi.z; ++z)
            for (int y = lo.y; y <= hi.y; ++y)
                for (int x = lo.x; x < hi.x; ++x) { /* exclusive upper x bound, cu:582 */
                    f3 v = vertex_pos((uint32_t)x, (uint32_t)y, (uint32_t)z, sc);
                    float dx = v.x - q.x, dy = v.y - q.y, dz = v.z - q.z;
                    float dist = sqrtf(dx * dx + dy * dy + dz * dz);
                    if ((double)dist < rad) {
                        uint32_t k = lin3((uint32_t)x, (uint32_t)y, (uint32_t)z, r);
#pragma omp atomic write
                        isSurf[k] = 1;
                    }
                }
    }
    return OK;
}

/* ------------------------------------------------------------------ */
/* ZB05 and TC01 fields (cu:178-289, 308-324; cuh:252-268)              */

/* kernelZB05: pow(1 - d2/h2, 3) with std::pow(float,int) promoting to double */
static inline real_t zb05_w(real_t d2, real_t h2)
{
    if (d2 >= h2) return 0;
#if FSR_REAL_BITS == 64
    real_t t = 1.0 - d2 / h2;
    return t * t * t;
#else
    float t = 1.0f - d2 / h2;
    return (float)pow((double)t, 3.0);
#endif
}

int o_field_zb05(const uint32_t* sv, uint32_t nb, const uint32_t* ranges, const float* pos,
                 uint32_t n, const o_gridinfo* sp, const o_gridinfo* sc, const o_simparam* p,
                 real_t* phi)
{
    (void)n;
    const real_t h2 = (real_t)p->smoothingRadiusSq;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)nb; ++t) {
        uint32_t x, y, z;
        unlin3(sv[t], sc->res, &x, &y, &z);
        f3 v = vertex_pos(x, y, z, sc);
        i3 c = cell_of(v, sp), lo, hi;
        window(c, 1, sp->res, &lo, &hi);
        real_t wsum = 0, ax = 0, ay = 0, az = 0;
        for (int zz = lo.z; zz <= hi.z; ++zz)
            for (int yy = lo.y; yy <= hi.y; ++yy)
                for (int xx = lo.x; xx <= hi.x; ++xx) {
                    uint32_t k = lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, sp->res);
                    uint32_t s = ranges[2 * k], e = ranges[2 * k + 1];
                    if (s == EMPTY_CELL) continue;
                    for (uint32_t i = s; i < e; ++i) {
                        f3 q = ld3(pos, i);
                        real_t dx = (real_t)v.x - (real_t)q.x, dy = (real_t)v.y - (real_t)q.y,
                               dz = (real_t)v.z - (real_t)q.z;
                        real_t d2 = dx * dx + dy * dy + dz * dz;
                        real_t w = zb05_w(d2, h2);
                        wsum += w;
                        ax += (real_t)q.x * w;
                        ay += (real_t)q.y * w;
                        az += (real_t)q.z * w;
                    }
                }
        if (wsum > 0) {
            ax /= wsum; ay /= wsum; az /= wsum;
            real_t dx = (real_t)v.x - ax, dy = (real_t)v.y - ay, dz = (real_t)v.z - az;
#if FSR_REAL_BITS == 64
            phi[sv[t]] = sqrt(dx * dx + dy * dy + dz * dz) - (real_t)p->particleRadius;
#else
            phi[sv[t]] = sqrtf(dx * dx + dy * dy + dz * dz) - p->particleRadius;
#endif
        }
    }
    return OK;
}

/* kernelTC01 (cuh:252-260): t = d2/h2*0.5, t^2 - t + 1/4, zero beyond h */
static inline real_t tc01_w(real_t d2, real_t h2)
{
    if (d2 > h2) return 0;
    real_t t = d2 / h2 * (real_t)0.5;
    real_t t2 = t * t;
    return t2 - t + (real_t)0.25;
}

int o_field_tc01(const uint32_t* sv, uint32_t nb, const uint32_t* ranges, const float* pos,
                 uint32_t n, const o_gridinfo* sp, const o_gridinfo* sc, const o_simparam* p,
                 real_t* phi)
{
    (void)n;
    const real_t h2 = (real_t)p->smoothingRadiusSq;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)nb; ++t) {
        uint32_t x, y, z;
        unlin3(sv[t], sc->res, &x, &y, &z);
        f3 v = vertex_pos(x, y, z, sc);
        i3 c = cell_of(v, sp), lo, hi;
        window(c, 1, sp->res, &lo, &hi);
        real_t val = 0;
        for (int zz = lo.z; zz <= hi.z; ++zz)
            for (int yy = lo.y; yy <= hi.y; ++yy)
                for (int xx = lo.x; xx <= hi.x; ++xx) {
                    uint32_t k = lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, sp->res);
                    uint32_t s = ranges[2 * k], e = ranges[2 * k + 1];
                    if (s == EMPTY_CELL) continue;
                    for (uint32_t i = s; i < e; ++i) {
                        f3 q = ld3(pos, i);
                        real_t dx = (real_t)v.x - (real_t)q.x, dy = (real_t)v.y - (real_t)q.y,
                               dz = (real_t)v.z - (real_t)q.z;
                        val += tc01_w(dx * dx + dy * dy + dz * dz, h2);
                    }
                }
        phi[sv[t]] = val;
    }
    return OK;
}

/* ------------------------------------------------------------------ */
/* anisotropic path: smoothing (cu:598-658)                              */

/* wij (cuh:282-292): 1 - (d/r)^3 inside r */
static inline float wij_f(float d, float r)
{
    if (d < r) {
        float s = d / r;
        return 1.0f - s * s * s;
    }
    return 0.0f;
}

static inline real_t wij_r(real_t d, real_t r)
{
    if (d < r) {
        real_t s = d / r;
        return (real_t)1 - s * s * s;
    }
    return 0;
}

/* Writes the FP32 mean (mean32, the reference's value, used for the FP32
 * neighbour-count decisions of the covariance stage) and the mean and
 * smoothed positions in real_t.  In the FP32 build mean and mean32 hold the
 * same numbers. */
int o_smooth2(const o_simparam* p, const float* pos, uint32_t n, const uint32_t* ranges,
              const o_gridinfo* sp, float* mean32, real_t* mean, real_t* smoothed)
{
    const float R = p->anisotropicRadius;
    const float lam = p->lambdaForSmoothed;
    const float one_minus = (float)(1.0 - (double)lam); /* (1.0 - lambda) promoted, cu:656 */
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)n; ++t) {
        f3 q = ld3(pos, (uint32_t)t);
        i3 c = cell_of(q, sp), lo, hi;
        window(c, 2, sp->res, &lo, &hi);
        float ws = 0.0f, mx = 0.0f, my = 0.0f, mz = 0.0f;
#if FSR_REAL_BITS == 64
        real_t wsr = 0, mxr = 0, myr = 0, mzr = 0;
#endif
        for (int zz = lo.z; zz <= hi.z; ++zz)
            for (int yy = lo.y; yy <= hi.y; ++yy)
                for (int xx = lo.x; xx <= hi.x; ++xx) {
                    uint32_t k = lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, sp->res);
                    uint32_t s = ranges[2 * k], e = ranges[2 * k + 1];
                    if (s == EMPTY_CELL) continue;
                    for (uint32_t i = s; i < e; ++i) {
                        f3 o = ld3(pos, i);
                        float dx = q.x - o.x, dy = q.y - o.y, dz = q.z - o.z;
                        float d = sqrtf(dx * dx + dy * dy + dz * dz);
                        float w = wij_f(d, R);
                        ws += w;
                        mx += o.x * w;
                        my += o.y * w;
                        mz += o.z * w;
#if FSR_REAL_BITS == 64
                        real_t ex = (real_t)q.x - o.x, ey = (real_t)q.y - o.y, ez = (real_t)q.z - o.z;
                        real_t wr = wij_r(sqrt(ex * ex + ey * ey + ez * ez), (real_t)R);
                        wsr += wr;
                        mxr += (real_t)o.x * wr;
                        myr += (real_t)o.y * wr;
                        mzr += (real_t)o.z * wr;
#endif
                    }
                }
        if (ws > 0.0f) { /* always true: the particle itself weighs 1 */
            mx /= ws; my /= ws; mz /= ws;
            mean32[3 * t] = mx; mean32[3 * t + 1] = my; mean32[3 * t + 2] = mz;
#if FSR_REAL_BITS == 64
            mxr /= wsr; myr /= wsr; mzr /= wsr;
            mean[3 * t] = mxr; mean[3 * t + 1] = myr; mean[3 * t + 2] = mzr;
            smoothed[3 * t] = (1.0 - (double)lam) * q.x + (double)lam * mxr;
            smoothed[3 * t + 1] = (1.0 - (double)lam) * q.y + (double)lam * myr;
            smoothed[3 * t + 2] = (1.0 - (double)lam) * q.z + (double)lam * mzr;
#else
            mean[3 * t] = mx; mean[3 * t + 1] = my; mean[3 * t + 2] = mz;
            smoothed[3 * t] = one_minus * q.x + lam * mx;
            smoothed[3 * t + 1] = one_minus * q.y + lam * my;
            smoothed[3 * t + 2] = one_minus * q.z + lam * mz;
#endif
        }
    }
    (void)one_minus;
    return OK;
}

/* Same call shape as the reference launcher (mean and smoothed only). */
int o_smooth(const o_simparam* p, const float* pos, uint32_t n, const uint32_t* ranges,
             const o_gridinfo* sp, real_t* mean, real_t* smoothed)
{
    float* m32 = (float*)malloc(sizeof(float) * 3 * (size_t)(n ? n : 1));
    if (!m32) return ERR_ARG;
    int rc = o_smooth2(p, pos, n, ranges, sp, m32, mean, smoothed);
    free(m32);
    return rc;
}

/* ------------------------------------------------------------------ */
/* symmetric 3x3 eigen-decomposition (cyclic Jacobi, FP64)              */

/* A = V diag(w) V^T for symmetric A (row-major a[3][3]); columns of v are
 * the eigenvectors.  Plain cyclic Jacobi rotations (Golub & Van Loan,
 * Matrix Computations, sec. 8.5) until the off-diagonal mass vanishes. */
static void jacobi3(const double a_in[3][3], double w[3], double v[3][3])
{
    double a[3][3];
    memcpy(a, a_in, sizeof(a));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off <= 1e-40 * diag || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (a[p][q] == 0.0) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) { /* A <- A J */
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) { /* A <- J^T A */
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 3; ++i) w[i] = a[i][i];
}

/* ------------------------------------------------------------------ */
/* anisotropic path: covariance and G (cu:689-827)                      */

/* mean32 carries the FP32 mean used for the neighbour-count decision
 * (dist <= r, cu:746); mean carries the mean the covariance is taken about. */
int o_cov2(const o_simparam* p, const o_gridinfo* sp, const float* mean32, const real_t* mean,
           const float* pos, uint32_t n, const uint32_t* ranges, const uint32_t* inv, uint32_t ni,
           real_t* G)
{
    (void)n;
    const float R = p->anisotropicRadius;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t t = 0; t < (int64_t)ni; ++t) {
        uint32_t pi = inv[t];
        f3 q = ld3(pos, pi);
        f3 m32 = ld3(mean32, pi);
        real_t mx = mean[3 * (size_t)pi], my = mean[3 * (size_t)pi + 1], mz = mean[3 * (size_t)pi + 2];
        i3 c = cell_of(q, sp), lo, hi;
        window(c, 2, sp->res, &lo, &hi);
        real_t a11, a22, a33, a12 = 0, a13 = 0, a21 = 0, a23 = 0, a31 = 0, a32 = 0;
        a11 = a22 = a33 = (real_t)p->smoothingRadiusSq;
        uint32_t nn = 0;
        real_t ws = 0;
        for (int zz = lo.z; zz <= hi.z; ++zz)
            for (int yy = lo.y; yy <= hi.y; ++yy)
                for (int xx = lo.x; xx <= hi.x; ++xx) {
                    uint32_t k = lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, sp->res);
                    uint32_t s = ranges[2 * k], e = ranges[2 * k + 1];
                    if (s == EMPTY_CELL) continue;
                    for (uint32_t i = s; i < e; ++i) {
                        f3 o = ld3(pos, i);
                        float fx = o.x - m32.x, fy = o.y - m32.y, fz = o.z - m32.z;
                        float fd = sqrtf(fx * fx + fy * fy + fz * fz);
                        if (fd <= R) ++nn;
#if FSR_REAL_BITS == 64
                        real_t vx = (real_t)o.x - mx, vy = (real_t)o.y - my, vz = (real_t)o.z - mz;
                        real_t w = wij_r(sqrt(vx * vx + vy * vy + vz * vz), (real_t)R);
#else
                        real_t vx = fx, vy = fy, vz = fz;
                        real_t w = wij_f(fd, R);
                        (void)mx; (void)my; (void)mz;
#endif
                        ws += w;
                        a11 += w * vx * vx;
                        a22 += w * vy * vy;
                        a33 += w * vz * vz;
                        real_t c12 = w * vx * vy, c13 = w * vx * vz, c23 = w * vy * vz;
                        a12 += c12; a21 += c12;
                        a13 += c13; a31 += c13;
                        a23 += c23; a32 += c23;
                    }
                }
        real_t* g = G + 9 * (size_t)t;
        if (nn < p->minNumNeighbors) { /* isolated particle: G = I / h */
            for (int k = 0; k < 9; ++k) g[k] = 0;
            g[0] = g[4] = g[8] = (real_t)p->smoothingRadiusInv;
            continue;
        }
        a11 /= ws; a12 /= ws; a13 /= ws;
        a21 /= ws; a22 /= ws; a23 /= ws;
        a31 /= ws; a32 /= ws; a33 /= ws;
        double A[3][3] = {{a11, a12, a13}, {a21, a22, a23}, {a31, a32, a33}};
        double w[3], V[3][3];
        jacobi3(A, w, V);
#if FSR_REAL_BITS == 64
        double s0 = fabs(w[0]), s1 = fabs(w[1]), s2 = fabs(w[2]);
        double smax = fmax(s0, fmax(s1, s2)) / 4.0;
        s0 = fmax(s0, smax); s1 = fmax(s1, smax); s2 = fmax(s2, smax);
        double inv_s[3] = {1.0 / s0, 1.0 / s1, 1.0 / s2};
        double cof = (1.0 / (double)p->smoothingRadius) * cbrt(s0 * s1 * s2);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double acc = 0.0;
                for (int k = 0; k < 3; ++k) acc += V[i][k] * inv_s[k] * V[j][k];
                g[3 * i + j] = acc * cof;
            }
#else
        /* the reference's post-SVD arithmetic (cu:790-822) in FP32 on the
         * FP32-rounded factors; U = W = V for a symmetric positive definite A */
        float u[3][3], sv[3];
        for (int i = 0; i < 3; ++i) {
            sv[i] = (float)w[i];
            for (int j = 0; j < 3; ++j) u[i][j] = (float)V[i][j];
        }
        float vx = fabsf(sv[0]), vy = fabsf(sv[1]), vz = fabsf(sv[2]);
        float msv = fmaxf(vx, fmaxf(vy, vz)) / 4.0f;
        vx = fmaxf(vx, msv); vy = fmaxf(vy, msv); vz = fmaxf(vz, msv);
        float ix = 1.0f / vx, iy = 1.0f / vy, iz = 1.0f / vz;
        /* ret = diag(1/sigma) U^T */
        float r11 = u[0][0] * ix, r12 = u[1][0] * ix, r13 = u[2][0] * ix;
        float r21 = u[0][1] * iy, r22 = u[1][1] * iy, r23 = u[2][1] * iy;
        float r31 = u[0][2] * iz, r32 = u[1][2] * iz, r33 = u[2][2] * iz;
        /* ret = W ret (matrixMul, cuh:664-687) */
        float c11 = u[0][0] * r11 + u[0][1] * r21 + u[0][2] * r31;
        float c21 = u[1][0] * r11 + u[1][1] * r21 + u[1][2] * r31;
        float c31 = u[2][0] * r11 + u[2][1] * r21 + u[2][2] * r31;
        float c12 = u[0][0] * r12 + u[0][1] * r22 + u[0][2] * r32;
        float c22 = u[1][0] * r12 + u[1][1] * r22 + u[1][2] * r32;
        float c32 = u[2][0] * r12 + u[2][1] * r22 + u[2][2] * r32;
        float c13 = u[0][0] * r13 + u[0][1] * r23 + u[0][2] * r33;
        float c23 = u[1][0] * r13 + u[1][1] * r23 + u[1][2] * r33;
        float c33 = u[2][0] * r13 + u[2][1] * r23 + u[2][2] * r33;
        float scale = powf(vx * vy * vz, (float)(1.0 / 3.0));
        float cof = p->smoothingRadiusInv * scale;
        g[0] = c11 * cof; g[1] = c12 * cof; g[2] = c13 * cof;
        g[3] = c21 * cof; g[4] = c22 * cof; g[5] = c23 * cof;
        g[6] = c31 * cof; g[7] = c32 * cof; g[8] = c33 * cof;
#endif
    }
    return OK;
}

int o_cov(const o_simparam* p, const o_gridinfo* sp, const real_t* mean, const float* pos,
          uint32_t n, const uint32_t* ranges, const uint32_t* inv, uint32_t ni, real_t* G)
{
#if FSR_REAL_BITS == 64
    (void)p; (void)sp; (void)mean; (void)pos; (void)n; (void)ranges; (void)inv; (void)ni; (void)G;
    return ERR_ARG; /* the FP64 build needs the FP32 mean: call o_cov2 */
#else
    return o_cov2(p, sp, mean, mean, pos, n, ranges, inv, ni, G);
#endif
}

/* ------------------------------------------------------------------ */
/* anisotropic field (cu:830-906; cuh:294-322, 689-700)                 */

static inline real_t det3(const real_t* m)
{
    return m[0] * m[4] * m[8] + m[1] * m[5] * m[6] + m[2] * m[3] * m[7] - m[0] * m[5] * m[7] -
           m[1] * m[3] * m[8] - m[2] * m[4] * m[6];
}

/* anisotropicW: |G r| via sqrt then squared, compared with 1.0 in double */
static inline real_t aniso_w(real_t rx, real_t ry, real_t rz, const real_t* g, real_t det)
{
    real_t tx = rx * g[0] + ry * g[1] + rz * g[2];
    real_t ty = rx * g[3] + ry * g[4] + rz * g[5];
    real_t tz = rx * g[6] + ry * g[7] + rz * g[8];
#if FSR_REAL_BITS == 64
    real_t d2 = tx * tx + ty * ty + tz * tz;
    if (d2 >= 1.0) return 0;
    real_t x = 1.0 - d2;
    return (315.0 / (64.0 * 3.14159265358979323846)) * det * x * x * x;
#else
    float dist = sqrtf(tx * tx + ty * ty + tz * tz);
    float d2 = dist * dist;
    if ((double)d2 >= 1.0) return 0.0f;
    float x = (float)(1.0 - (double)d2);
    return SIGMA_F * det * x * x * x;
#endif
}

/* anisotropicWOpt: the unscaled kernel of non-involved particles */
static inline real_t aniso_w_plain(real_t rx, real_t ry, real_t rz)
{
#if FSR_REAL_BITS == 64
    real_t d2 = rx * rx + ry * ry + rz * rz;
    if (d2 >= 1.0) return 0;
    real_t x = 1.0 - d2;
    return (315.0 / (64.0 * 3.14159265358979323846)) * x * x * x;
#else
    float dist = sqrtf(rx * rx + ry * ry + rz * rz);
    float d2 = dist * dist;
    if ((double)d2 >= 1.0) return 0.0f;
    float x = (float)(1.0 - (double)d2);
    return SIGMA_F * x * x * x;
#endif
}

int o_field_aniso(const o_simparam* p, uint32_t nb, const o_gridinfo* sc, const o_gridinfo* sp,
                  const real_t* G, uint32_t ni, const real_t* smoothed, const float* dens, uint32_t n,
                  const uint32_t* ranges, const uint32_t* sv, const uint32_t* ninv,
                  const uint32_t* ninvScan, real_t* phi)
{
    (void)ni; (void)n;
    const real_t mass = (real_t)p->particleMass;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t t = 0; t < (int64_t)nb; ++t) {
        uint32_t x, y, z;
        unlin3(sv[t], sc->res, &x, &y, &z);
        f3 v = vertex_pos(x, y, z, sc);
        i3 c = cell_of(v, sp), lo, hi;
        window(c, 2, sp->res, &lo, &hi);
        real_t sum = 0;
        for (int zz = lo.z; zz <= hi.z; ++zz)
            for (int yy = lo.y; yy <= hi.y; ++yy)
                for (int xx = lo.x; xx <= hi.x; ++xx) {
                    uint32_t k = lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, sp->res);
                    uint32_t s = ranges[2 * k], e = ranges[2 * k + 1];
                    if (ninv[k] > 0) {
                        uint32_t g0 = ninvScan[k];
                        for (uint32_t i = 0; i < e - s; ++i) {
                            const real_t* g = G + 9 * (size_t)(g0 + i);
                            const real_t* q = smoothed + 3 * (size_t)(s + i);
                            real_t w = aniso_w(q[0] - (real_t)v.x, q[1] - (real_t)v.y,
                                               q[2] - (real_t)v.z, g, det3(g));
                            sum += mass / (real_t)dens[s + i] * w;
                        }
                    } else {
                        if (s == EMPTY_CELL) continue;
                        for (uint32_t i = 0; i < e - s; ++i) {
                            const real_t* q = smoothed + 3 * (size_t)(s + i);
                            real_t w = aniso_w_plain(q[0] - (real_t)v.x, q[1] - (real_t)v.y,
                                                     q[2] - (real_t)v.z);
                            sum += mass / (real_t)dens[s + i] * w;
                        }
                    }
                }
        phi[sv[t]] = sum - (real_t)0.5;
    }
    return OK;
}

/* ------------------------------------------------------------------ */
/* Akinci12 colour-field surface test (cu:909-971; cuh:324-334)          */

int o_colorfield(const o_simparam* p, const float* pos, const float* dens, uint32_t n,
                 const uint32_t* ranges, const o_gridinfo* sp, uint32_t* sflag)
{
    const float h = p->smoothingRadius, h2 = p->smoothingRadiusSq, m = p->particleMass;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)n; ++t) {
        f3 q = ld3(pos, (uint32_t)t);
        i3 c = cell_of(q, sp), lo, hi;
        window(c, 1, sp->res, &lo, &hi);
        uint32_t nn = 0;
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        for (int zz = lo.z; zz <= hi.z; ++zz)
            for (int yy = lo.y; yy <= hi.y; ++yy)
                for (int xx = lo.x; xx <= hi.x; ++xx) {
                    uint32_t k = lin3((uint32_t)xx, (uint32_t)yy, (uint32_t)zz, sp->res);
                    uint32_t s = ranges[2 * k], e = ranges[2 * k + 1];
                    if (s == EMPTY_CELL) continue;
                    for (uint32_t i = s; i < e; ++i) {
                        f3 o = ld3(pos, i);
                        float rx = q.x - o.x, ry = q.y - o.y, rz = q.z - o.z;
                        float d2 = rx * rx + ry * ry + rz * rz;
                        if (!(d2 > 0.0f)) continue;
                        ++nn;
                        /* wSpikyGrad: -45/(pi h^4) (1 - d/h)^2 in double */
                        float d = sqrtf(d2);
                        float grad = 0.0f;
                        if (!(d >= h)) {
                            float x = (float)(1.0 - (double)(d / h));
                            grad = (float)(-45.0 / (3.1415926535 * (double)h2 * (double)h2) *
                                           (double)x * (double)x);
                        }
                        float inv = 1.0f / sqrtf(d2); /* normalize, host rsqrtf */
                        rx *= inv; ry *= inv; rz *= inv;
                        float coef = m / dens[i] * grad;
                        sx += coef * rx;
                        sy += coef * ry;
                        sz += coef * rz;
                    }
                }
        if (nn < 25) {
            sflag[t] = 1;
        } else if (sqrtf(sx * sx + sy * sy + sz * sz) > 3.0f) {
            sflag[t] = 1;
        }
    }
    return OK;
}

/* ------------------------------------------------------------------ */
/* marching cubes: classify (cu:328-364, 974-1008; cuh:534-544, 602-609) */

static inline void cube_corners(uint32_t x, uint32_t y, uint32_t z, const uint32_t r[3], uint32_t c[8])
{
    for (int i = 0; i < 8; ++i)
        c[i] = lin3(x + (uint32_t)FSR_O_CORNER[i][0], y + (uint32_t)FSR_O_CORNER[i][1],
                    z + (uint32_t)FSR_O_CORNER[i][2], r);
}

static int classify_one(uint32_t cube, const real_t* phi, const o_gridinfo* sc,
                        const uint32_t* isSurf, real_t iso, uint32_t* caseOut)
{
    const uint32_t* r = sc->res;
    uint32_t x, y, z;
    unlin3(cube, r, &x, &y, &z);
    if (x >= r[0] - 1 || y >= r[1] - 1 || z >= r[2] - 1) return -1;
    uint32_t c[8];
    cube_corners(x, y, z, r, c);
    uint32_t f = 0;
    for (int i = 0; i < 8; ++i)
        if (phi[c[i]] <= iso) f |= 1u << i;
    *caseOut = f;
    for (int i = 0; i < 8; ++i)
        if (!isSurf[c[i]]) return 0;
    return 1;
}

int o_classify(const uint32_t* sv, uint32_t nb, const real_t* phi, const o_gridinfo* sc,
               const uint32_t* isSurf, const o_simparam* p, uint32_t* valid, uint32_t* nverts)
{
    const real_t iso = (real_t)p->isoValue;
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < (int64_t)nb; ++t) {
        uint32_t f = 0;
        int all = classify_one(sv[t], phi, sc, isSurf, iso, &f);
        if (all < 0) continue;
        uint32_t nv = all ? fsr_o_num_vertices(f) : 0;
        valid[t] = nv > 0 ? 1 : 0;
        nverts[t] = nv;
    }
    return OK;
}

int o_classify_akinci(const uint32_t* sv, uint32_t nb, const real_t* phi, const o_gridinfo* sc,
                      const uint32_t* isSurf, const o_simparam* p, uint32_t* valid)
{
    const real_t iso = (real_t)p->isoValue;
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < (int64_t)nb; ++t) {
        uint32_t f = 0;
        int all = classify_one(sv[t], phi, sc, isSurf, iso, &f);
        if (all < 0) continue;
        uint32_t nv = all ? fsr_o_num_vertices(f) : 0;
        valid[t] = nv > 0 ? 1 : 0;
    }
    return OK;
}

/* The MC case of each listed cube (diagnostics: case-index parity). */
int o_cases(const uint32_t* cubes, uint32_t nq, const real_t* phi, const o_gridinfo* sc,
            const o_simparam* p, uint32_t* cases)
{
    const real_t iso = (real_t)p->isoValue;
    for (uint32_t t = 0; t < nq; ++t) {
        uint32_t x, y, z, c[8], f = 0;
        unlin3(cubes[t], sc->res, &x, &y, &z);
        cube_corners(x, y, z, sc->res, c);
        for (int i = 0; i < 8; ++i)
            if (phi[c[i]] <= iso) f |= 1u << i;
        cases[t] = f;
    }
    return OK;
}

/* ------------------------------------------------------------------ */
/* marching cubes: generation (cu:383-463; cuh:372-379, 410-430)         */

static inline real_t grid_value(int x, int y, int z, const real_t* phi, const uint32_t r[3])
{
    if (x < 0 || y < 0 || z < 0 || (uint32_t)x >= r[0] || (uint32_t)y >= r[1] || (uint32_t)z >= r[2])
        return 0;
    return phi[lin3((uint32_t)x, (uint32_t)y, (uint32_t)z, r)];
}

/* normalize(): v * rsqrt(dot(v,v)), host rsqrtf = 1/sqrtf */
static inline void normalize_gpu(real_t* n)
{
#if FSR_REAL_BITS == 64
    real_t inv = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
#else
    float inv = 1.0f / sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
#endif
    n[0] *= inv; n[1] *= inv; n[2] *= inv;
}

static inline void corner_normal(int x, int y, int z, const real_t* phi, const uint32_t r[3], real_t n[3])
{
    n[0] = grid_value(x - 1, y, z, phi, r) - grid_value(x + 1, y, z, phi, r);
    n[1] = grid_value(x, y - 1, z, phi, r) - grid_value(x, y + 1, z, phi, r);
    n[2] = grid_value(x, y, z - 1, phi, r) - grid_value(x, y, z + 1, phi, r);
}

static inline real_t lerp_fac_gpu(real_t a, real_t b, real_t iso)
{
    real_t d = b - a;
    if (d > (real_t)EPS_F * -1 && d < (real_t)EPS_F) return (real_t)0.5;
    return (iso - a) / d;
}

/* o_generate plus, per mesh vertex, the length of the interpolated normal
 * before its normalisation (outLen, may be NULL): directions of short
 * interpolated normals are ill-conditioned, which the tests account for. */
int o_generate2(const uint32_t* sv, uint32_t nb, const uint32_t* validIdx, uint32_t nq,
                const o_gridinfo* sc, const uint32_t* nvScan, const real_t* phi, const o_simparam* p,
                real_t* outPos, real_t* outNrm, real_t* outLen, uint64_t nOut)
{
    (void)nb;
    const real_t iso = (real_t)p->isoValue;
    const real_t sgn = p->isoValue < 0.0f ? (real_t)-1 : (real_t)1;
    const uint32_t* r = sc->res;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : bad)
    for (int64_t q = 0; q < (int64_t)nq; ++q) {
        uint32_t s = validIdx[q];
        uint32_t x, y, z;
        unlin3(sv[s], r, &x, &y, &z);
        real_t val[8], cp[8][3], cn[8][3];
        uint32_t f = 0;
        for (int i = 0; i < 8; ++i) {
            int cx = (int)x + FSR_O_CORNER[i][0], cy = (int)y + FSR_O_CORNER[i][1],
                cz = (int)z + FSR_O_CORNER[i][2];
            val[i] = grid_value(cx, cy, cz, phi, r);
            if (val[i] <= iso) f |= 1u << i;
            f3 pv = vertex_pos((uint32_t)cx, (uint32_t)cy, (uint32_t)cz, sc);
            cp[i][0] = pv.x; cp[i][1] = pv.y; cp[i][2] = pv.z;
            corner_normal(cx, cy, cz, phi, r, cn[i]);
            normalize_gpu(cn[i]);
        }
        uint32_t ef = fsr_o_edge_flags(f), nv = fsr_o_num_vertices(f);
        real_t ip[12][3], in[12][3], il[12];
        for (int e = 0; e < 12; ++e) {
            if (!(ef & (1u << e))) continue;
            int a = FSR_O_EDGE[e][0], b = FSR_O_EDGE[e][1];
            real_t t = lerp_fac_gpu(val[a], val[b], iso);
            for (int k = 0; k < 3; ++k) {
                ip[e][k] = cp[a][k] + t * (cp[b][k] - cp[a][k]);
                in[e][k] = cn[a][k] + t * (cn[b][k] - cn[a][k]);
            }
            il[e] = sqrt((double)(in[e][0] * in[e][0] + in[e][1] * in[e][1] + in[e][2] * in[e][2]));
            normalize_gpu(in[e]);
            for (int k = 0; k < 3; ++k) in[e][k] = sgn * in[e][k];
        }
        uint64_t base = nvScan[s];
        if (base + nv > nOut) { bad |= 1; continue; }
        for (uint32_t k = 0; k < nv; ++k) {
            int e = fsr_o_tri_edge(f, k);
            for (int j = 0; j < 3; ++j) {
                outPos[3 * (base + k) + j] = ip[e][j];
                outNrm[3 * (base + k) + j] = in[e][j];
            }
            if (outLen) outLen[base + k] = il[e];
        }
    }
    return bad ? ERR_ARG : OK;
}

int o_generate(const uint32_t* sv, uint32_t nb, const uint32_t* validIdx, uint32_t nq,
               const o_gridinfo* sc, const uint32_t* nvScan, const real_t* phi, const o_simparam* p,
               real_t* outPos, real_t* outNrm, uint64_t nOut)
{
    return o_generate2(sv, nb, validIdx, nq, sc, nvScan, phi, p, outPos, outNrm, NULL, nOut);
}

/* ------------------------------------------------------------------ */
/* Akinci12's host marching cubes (MarchingCubesCPU.cpp:3-89, .h:104-177) */

static inline void normalize_host(real_t* n) /* fVector3::normalize, MathVector.cpp:5-15 */
{
#if FSR_REAL_BITS == 64
    real_t len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
#else
    float len = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
#endif
    if (len > (real_t)(float)1.0e-7) {
        real_t fac = (real_t)1 / len;
        n[0] *= fac; n[1] *= fac; n[2] *= fac;
    }
}

int64_t o_mc_cpu2(const real_t* phi, const o_gridinfo* sc, float iso_f, const uint32_t* cubeVertex,
                  uint32_t nq, real_t* outPos, real_t* outNrm, real_t* outLen, uint64_t capacity)
{
    const uint32_t* r = sc->res;
    const real_t iso = (real_t)iso_f;
    uint64_t out = 0;
    for (uint32_t q = 0; q < nq; ++q) {
        uint32_t x, y, z;
        unlin3(cubeVertex[q], r, &x, &y, &z);
        real_t val[8], cp[8][3], cn[8][3];
        uint32_t f = 0;
        for (int i = 0; i < 8; ++i) {
            int cx = (int)x + FSR_O_CORNER[i][0], cy = (int)y + FSR_O_CORNER[i][1],
                cz = (int)z + FSR_O_CORNER[i][2];
            val[i] = grid_value(cx, cy, cz, phi, r);
            cp[i][0] = sc->minPos[0] + (float)cx * sc->cellSize;
            cp[i][1] = sc->minPos[1] + (float)cy * sc->cellSize;
            cp[i][2] = sc->minPos[2] + (float)cz * sc->cellSize;
            corner_normal(cx, cy, cz, phi, r, cn[i]);
            normalize_host(cn[i]);
            if (val[i] <= iso) f |= 1u << i;
        }
        if (f == 0 || f == 255) continue;
        uint32_t ef = fsr_o_edge_flags(f), nv = fsr_o_num_vertices(f);
        real_t ip[12][3], in[12][3], il[12];
        for (int e = 0; e < 12; ++e) {
            if (!(ef & (1u << e))) continue;
            int a = FSR_O_EDGE[e][0], b = FSR_O_EDGE[e][1];
            real_t d = val[b] - val[a];
            real_t t = (d > -1.0e-7 && d < 1.0e-7) ? (real_t)0.5 : (iso - val[a]) / d;
            for (int k = 0; k < 3; ++k) {
                ip[e][k] = cp[a][k] + (cp[b][k] - cp[a][k]) * t;
                in[e][k] = cn[a][k] + (cn[b][k] - cn[a][k]) * t;
            }
            il[e] = sqrt((double)(in[e][0] * in[e][0] + in[e][1] * in[e][1] + in[e][2] * in[e][2]));
            normalize_host(in[e]);
        }
        if (out + nv > capacity) return -1;
        for (uint32_t k = 0; k < nv; ++k) {
            int e = fsr_o_tri_edge(f, k);
            for (int j = 0; j < 3; ++j) {
                outPos[3 * (out + k) + j] = ip[e][j];
                outNrm[3 * (out + k) + j] = in[e][j];
            }
            if (outLen) outLen[out + k] = il[e];
        }
        out += nv;
    }
    return (int64_t)out;
}

int64_t o_mc_cpu(const real_t* phi, const o_gridinfo* sc, float iso_f, const uint32_t* cubeVertex,
                 uint32_t nq, real_t* outPos, real_t* outNrm, uint64_t capacity)
{
    return o_mc_cpu2(phi, sc, iso_f, cubeVertex, nq, outPos, outNrm, NULL, capacity);
}
