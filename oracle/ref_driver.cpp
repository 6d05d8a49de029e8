/*
 * Host launcher for the reference's own CUDA kernel bodies, compiled as C++
 * (oracle recipe: oracle/build_ref.sh).  TEST INFRASTRUCTURE ONLY.
 *
 * The kernel bodies are not part of this repository: the recipe extracts
 * them at build time from FluidSurfaceReconstruction/GPU/ReconstructionCUDA.cu
 * (lines 28-1008 and 1354-1396, i.e. every __global__/__device__ kernel
 * except findCellRangeKernel, which needs shared memory and a barrier) into
 * oracle/_ref/ref_kernels.inc, which is included below.
 *
 * Each o_* function below reproduces one launch of the reference's host code:
 * the thread domain and block shape come from calcGridDimBlockDim
 * (GPU/CudaUtils.h:87-106: 128-thread blocks, grid spilling into y above
 * 65,535 blocks) or from launchSpatialGridBuilding (ReconstructionCUDA.cu:
 * 1450-1456: 256-thread blocks).  Logical threads run in an OpenMP loop with
 * the launch coordinates set per OS thread.
 *
 * Two deliberate deviations:
 *  - the smoothing kernel (ReconstructionCUDA.cu:609, bound "threadId >
 *    size") is run over exactly N threads, so the out-of-bounds thread N
 *    never executes;
 *  - thrust::sort_by_key / exclusive_scan / findCellRangeKernel are not
 *    emulated here: their results are defined exactly (stable sort, prefix
 *    sum, segment bounds) and the Python composition computes them.
 */
#include "fsr_ref_emul.h"

#include "ReconstructionCUDA.cuh"
#include "SVD3.cuh"
#include "MarchingCubesHelper.h"
#include "MarchingCubesCPU.h"

#include "fsr_stage_api.h"

#include <omp.h>
#include <cstring>
#include <vector>

thread_local uint3 blockIdx;
thread_local uint3 threadIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

/* The two __constant__ definitions of ReconstructionCUDA.cu:25-26. */
extern "C" float EPSILON_ = (float)1.0e-7;
extern "C" float SIGMA = 315.0f / (64.0f * 3.1415926535898f);

/* Only referenced by bindTextures(); the channel format is irrelevant here. */
extern "C" cudaChannelFormatDesc cudaCreateChannelDesc(int x, int y, int z, int w,
                                                       enum cudaChannelFormatKind f)
{
    cudaChannelFormatDesc d;
    d.x = x; d.y = y; d.z = z; d.w = w; d.f = f;
    return d;
}

#include "ref_kernels.inc"

namespace {

/* Runs body() once per logical thread of a <<<grid, block>>> launch whose
 * linear thread count is blocks*threadsPerBlock, with the grid shaped the way
 * the reference's host code shapes it. */
template <class Body>
void launch(uint64_t blocks, unsigned threadsPerBlock, bool spillY, Body body)
{
    if (blocks == 0) return;
    dim3 g((unsigned)blocks, 1, 1);
    if (spillY && blocks > 65535) {
        g.x = 65535;
        g.y = (unsigned)((blocks + 65534) / 65535);
    }
    const dim3 b(threadsPerBlock, 1, 1);
    const int64_t total = (int64_t)(blocks * threadsPerBlock);
#pragma omp parallel for schedule(dynamic, 2048)
    for (int64_t t = 0; t < total; ++t) {
        const uint64_t bid = (uint64_t)t / threadsPerBlock;
        blockIdx = make_uint3((unsigned)(bid % g.x), (unsigned)(bid / g.x), 0);
        threadIdx = make_uint3((unsigned)(t % threadsPerBlock), 0, 0);
        blockDim = b;
        gridDim = g;
        body();
    }
}

/* calcGridDimBlockDim(threadSize): ceil(threadSize/128) blocks of 128. */
template <class Body>
void launch128(uint64_t threadSize, Body body)
{
    launch((threadSize + 127) / 128, 128, true, body);
}

GridInfo toGridInfo(const o_gridinfo* g)
{
    GridInfo r;
    r.minPos = make_float3(g->minPos[0], g->minPos[1], g->minPos[2]);
    r.maxPos = make_float3(g->maxPos[0], g->maxPos[1], g->maxPos[2]);
    r.cellSize = g->cellSize;
    r.resolution = make_uint3(g->res[0], g->res[1], g->res[2]);
    return r;
}

SimParam toSimParam(const o_simparam* p)
{
    static_assert(sizeof(SimParam) == sizeof(o_simparam), "SimParam layout");
    SimParam s;
    std::memcpy(&s, p, sizeof(s));
    return s;
}

template <class T>
Grid<T> grid3(T* ptr, const o_gridinfo* g)
{
    Grid<T> r;
    r.grid = ptr;
    r.resolution = make_uint3(g->res[0], g->res[1], g->res[2]);
    r.size = (unsigned long long)g->res[0] * g->res[1] * g->res[2];
    r.count = r.size;
    return r;
}

template <class T>
Grid<T> grid1(T* ptr, uint64_t n)
{
    Grid<T> r;
    r.grid = ptr;
    r.resolution = make_uint3((unsigned)n, 1, 1);
    r.size = n;
    r.count = n;
    return r;
}

struct TablesBound {
    TablesBound()
    {
        bindTextures(const_cast<uint*>(MarchingCubesHelper::edgeFlags),
                     const_cast<int*>(&MarchingCubesHelper::edgeIndexesOfTriangle[0][0]),
                     const_cast<uint*>(MarchingCubesHelper::numVertices),
                     const_cast<uint*>(&MarchingCubesHelper::vertexIndexesOfEdge[0][0]));
    }
};

void bindOnce() { static TablesBound once; }

} // namespace

extern "C" {

int o_real_bytes(void) { return 4; }
int o_is_reference(void) { return 1; }
int o_set_threads(int n) { if (n > 0) omp_set_num_threads(n); return omp_get_max_threads(); }

/* calcParticlesHashKernel, launched as launchSpatialGridBuilding does. */
int o_hash(const float* pos, uint32_t n, const o_gridinfo* sp, uint32_t* keys, float* flag)
{
    ParticleArray parts = grid1((ParticlePosition*)pos, n);
    DensityGrid fg = grid3(flag, sp);
    GridInfo gi = toGridInfo(sp);
    launch((n + 255) / 256, 256, false, [&] { calcParticlesHashKernel(keys, parts, n, fg, gi); });
    return 0;
}

int o_surface(const o_simparam* p, const float* flag, const uint32_t* ranges,
              const o_gridinfo* sp, uint32_t* sflag, uint32_t n)
{
    SimParam s = toSimParam(p);
    DensityGrid fg = grid3((float*)flag, sp);
    IsSurfaceGrid sf = grid1(sflag, n);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    launch128(rg.size, [&] { extractionOfSurfaceParticles(s, fg, sf, rg); });
    return 0;
}

int o_surface_involve(const o_simparam* p, const float* flag, const uint32_t* ranges,
                      const o_gridinfo* sp, uint32_t* sflag, uint32_t n, uint32_t* ninv)
{
    SimParam s = toSimParam(p);
    DensityGrid fg = grid3((float*)flag, sp);
    IsSurfaceGrid sf = grid1(sflag, n);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    NumInvolveParticlesGrid ni = grid3(ninv, sp);
    launch128(rg.size, [&] { extractionOfSurfaceAndInvolveParticles(s, fg, ni, sf, rg); });
    return 0;
}

int o_band(const o_simparam* p, const o_gridinfo* sc, const float* pos, const uint32_t* sflag,
           uint32_t n, const uint32_t* ranges, const o_gridinfo* sp, uint32_t* isSurf)
{
    SimParam s = toSimParam(p);
    GridInfo sci = toGridInfo(sc);
    ParticleArray parts = grid1((ParticlePosition*)pos, n);
    IsSurfaceGrid sf = grid1((uint*)sflag, n);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    IsSurfaceGrid band = grid3(isSurf, sc);
    launch128(n, [&] { estimationOfSurfaceVertices(s, sci, parts, sf, rg, band); });
    return 0;
}

int o_field_zb05(const uint32_t* sv, uint32_t nb, const uint32_t* ranges, const float* pos,
                 uint32_t n, const o_gridinfo* sp, const o_gridinfo* sc, const o_simparam* p,
                 float* phi)
{
    SimParam s = toSimParam(p);
    SurfaceVerticesIndexArray svi = grid1((uint*)sv, nb);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    ParticleArray parts = grid1((ParticlePosition*)pos, n);
    ScalarFieldGrid field = grid3((ScalarValue*)phi, sc);
    GridInfo spi = toGridInfo(sp), sci = toGridInfo(sc);
    launch128(nb, [&] { updateScalarGridValuesCompacted(svi, nb, rg, parts, field, spi, sci, s); });
    return 0;
}

/* TC01 has no launcher in the reference: the device function
 * updateScalarFieldValueTC01 (ReconstructionCUDA.cu:178-227) is driven the
 * way updateScalarGridValuesCompacted drives its ZB05 sibling. */
int o_field_tc01(const uint32_t* sv, uint32_t nb, const uint32_t* ranges, const float* pos,
                 uint32_t n, const o_gridinfo* sp, const o_gridinfo* sc, const o_simparam* p,
                 float* phi)
{
    SimParam s = toSimParam(p);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    ParticleArray parts = grid1((ParticlePosition*)pos, n);
    ScalarFieldGrid field = grid3((ScalarValue*)phi, sc);
    GridInfo spi = toGridInfo(sp), sci = toGridInfo(sc);
    launch128(nb, [&] {
        uint t = blockIdx.x * 128 + threadIdx.x + blockIdx.y * gridDim.x * 128;
        if (t < nb) updateScalarFieldValueTC01(sv[t], rg, parts, field, spi, sci, s);
    });
    return 0;
}

int o_smooth(const o_simparam* p, const float* pos, uint32_t n, const uint32_t* ranges,
             const o_gridinfo* sp, float* mean, float* smoothed)
{
    SimParam s = toSimParam(p);
    ParticleArray parts = grid1((ParticlePosition*)pos, n);
    ParticleArray m = grid1((ParticlePosition*)mean, n);
    ParticleArray sm = grid1((ParticlePosition*)smoothed, n);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    GridInfo spi = toGridInfo(sp);
    /* exactly n logical threads: see the header comment (bound at cu:609) */
    if (n == 0) return 0;
    const dim3 b(128, 1, 1);
    const uint64_t blocks = (n + 127) / 128;
    dim3 g((unsigned)blocks, 1, 1);
    if (blocks > 65535) { g.x = 65535; g.y = (unsigned)((blocks + 65534) / 65535); }
#pragma omp parallel for schedule(dynamic, 2048)
    for (int64_t t = 0; t < (int64_t)n; ++t) {
        const uint64_t bid = (uint64_t)t / 128;
        blockIdx = make_uint3((unsigned)(bid % g.x), (unsigned)(bid / g.x), 0);
        threadIdx = make_uint3((unsigned)(t % 128), 0, 0);
        blockDim = b;
        gridDim = g;
        calculationOfMeanAndSmoothParticles(s, parts, m, sm, rg, spi);
    }
    return 0;
}

int o_cov(const o_simparam* p, const o_gridinfo* sp, const float* mean, const float* pos,
          uint32_t n, const uint32_t* ranges, const uint32_t* inv, uint32_t ni, float* G)
{
    SimParam s = toSimParam(p);
    GridInfo spi = toGridInfo(sp);
    ParticleArray m = grid1((ParticlePosition*)mean, n);
    ParticleArray parts = grid1((ParticlePosition*)pos, n);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    SurfaceParticlesIndexArray ia = grid1((uint*)inv, ni);
    MatrixArray mats = grid1((MatrixValue*)G, ni);
    launch128(ni, [&] { calculationOfTransformMatricesForParticles(s, spi, m, parts, rg, ia, mats); });
    return 0;
}

int o_field_aniso(const o_simparam* p, uint32_t nb, const o_gridinfo* sc, const o_gridinfo* sp,
                  const float* G, uint32_t ni, const float* smoothed, const float* dens, uint32_t n,
                  const uint32_t* ranges, const uint32_t* sv, const uint32_t* ninv,
                  const uint32_t* ninvScan, float* phi)
{
    SimParam s = toSimParam(p);
    GridInfo sci = toGridInfo(sc), spi = toGridInfo(sp);
    MatrixArray mats = grid1((MatrixValue*)G, ni);
    ParticleArray sm = grid1((ParticlePosition*)smoothed, n);
    ScalarFieldGrid d = grid1((ScalarValue*)dens, n);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    SurfaceVerticesIndexArray svi = grid1((uint*)sv, nb);
    NumInvolveParticlesGrid nig = grid3((uint*)ninv, sp);
    NumInvolveParticlesGrid nis = grid3((uint*)ninvScan, sp);
    ScalarFieldGrid field = grid3((ScalarValue*)phi, sc);
    launch128(nb, [&] {
        computationOfScalarFieldGrid(s, nb, sci, spi, mats, sm, d, rg, svi, nig, nis, field);
    });
    return 0;
}

int o_colorfield(const o_simparam* p, const float* pos, const float* dens, uint32_t n,
                 const uint32_t* ranges, const o_gridinfo* sp, uint32_t* sflag)
{
    SimParam s = toSimParam(p);
    ParticleArray parts = grid1((ParticlePosition*)pos, n);
    ScalarFieldGrid d = grid1((ScalarValue*)dens, n);
    ParticleIndexRangeGrid rg = grid3((IndexRange*)ranges, sp);
    GridInfo spi = toGridInfo(sp);
    IsSurfaceGrid sf = grid1(sflag, n);
    launch128(n, [&] { extractionOfSurfaceParticlesUsingColorField(s, parts, d, rg, spi, sf); });
    return 0;
}

int o_classify(const uint32_t* sv, uint32_t nb, const float* phi, const o_gridinfo* sc,
               const uint32_t* isSurf, const o_simparam* p, uint32_t* valid, uint32_t* nverts)
{
    bindOnce();
    SimParam s = toSimParam(p);
    SurfaceVerticesIndexArray svi = grid1((uint*)sv, nb);
    ScalarFieldGrid field = grid3((ScalarValue*)phi, sc);
    IsValidSurfaceGrid vg = grid1(valid, nb);
    NumVerticesGrid nvg = grid1(nverts, nb);
    IsSurfaceGrid band = grid3((uint*)isSurf, sc);
    launch128(nb, [&] { detectValidSurfaceCubes(svi, nb, field, vg, nvg, band, s); });
    return 0;
}

int o_classify_akinci(const uint32_t* sv, uint32_t nb, const float* phi, const o_gridinfo* sc,
                      const uint32_t* isSurf, const o_simparam* p, uint32_t* valid)
{
    bindOnce();
    SimParam s = toSimParam(p);
    SurfaceVerticesIndexArray svi = grid1((uint*)sv, nb);
    ScalarFieldGrid field = grid3((ScalarValue*)phi, sc);
    IsValidSurfaceGrid vg = grid1(valid, nb);
    IsSurfaceGrid band = grid3((uint*)isSurf, sc);
    launch128(nb, [&] { detectionOfValidSurfaceCubesForAkinci(svi, nb, field, vg, band, s); });
    return 0;
}

int o_generate(const uint32_t* sv, uint32_t nb, const uint32_t* validIdx, uint32_t nq,
               const o_gridinfo* sc, const uint32_t* nvScan, const float* phi, const o_simparam* p,
               float* outPos, float* outNrm, uint64_t nOut)
{
    bindOnce();
    SimParam s = toSimParam(p);
    SurfaceVerticesIndexArray svi = grid1((uint*)sv, nb);
    ValidSurfaceIndexArray vi = grid1((uint*)validIdx, nq);
    GridInfo sci = toGridInfo(sc);
    NumVerticesGrid nvs = grid1((uint*)nvScan, nb);
    ScalarFieldGrid field = grid3((ScalarValue*)phi, sc);
    Float3Grid pg = grid1((float3*)outPos, nOut);
    Float3Grid ng = grid1((float3*)outNrm, nOut);
    launch128(nq, [&] { generateTriangles(svi, vi, sci, nvs, field, pg, ng, s); });
    return 0;
}

/* Akinci12's host marching cubes (ReconstructorGPUAkinci12.cpp:262-287),
 * run with the reference's MarchingCubesCPU class.  Returns the number of
 * mesh vertices written, or -1 when the output capacity is too small. */
int64_t o_mc_cpu(const float* phi, const o_gridinfo* sc, float iso, const uint32_t* cubeVertex,
                 uint32_t nq, float* outPos, float* outNrm, uint64_t capacity)
{
    const uint64_t v = (uint64_t)sc->res[0] * sc->res[1] * sc->res[2];
    std::vector<ScalarValue> grid(v);
    std::memcpy(grid.data(), phi, v * sizeof(float));
    MarchingCubesCPU mc(&grid, toGridInfo(sc), iso);
    uint64_t out = 0;
    for (uint32_t q = 0; q < nq; ++q) {
        iVector3 idx = mc.index1DTo3D((int)cubeVertex[q]);
        Triangle tris[5];
        int count = 0;
        mc.marchingCubes(idx, tris, count);
        for (int t = 0; t < count; ++t) {
            for (int k = 0; k < 3; ++k) {
                if (out >= capacity) return -1;
                outPos[3 * out + 0] = tris[t].vertices[k].x;
                outPos[3 * out + 1] = tris[t].vertices[k].y;
                outPos[3 * out + 2] = tris[t].vertices[k].z;
                outNrm[3 * out + 0] = tris[t].normals[k].x;
                outNrm[3 * out + 1] = tris[t].normals[k].y;
                outNrm[3 * out + 2] = tris[t].normals[k].z;
                ++out;
            }
        }
    }
    return (int64_t)out;
}

} // extern "C"
