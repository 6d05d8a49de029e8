// Test helper: calls the reference-ABI launchers of a library from C++
// with by-value structs, exactly as the reference's host classes do, behind
// wrappers that take pointers (so Python never passes large structs by
// value through ctypes).  Compiled by oracle/ref_gpu/flow.py against
// libfsr_gb300.so (the compatibility layer, csrc/compat.cu) or against
// oracle/_build/libref_gpu.so (the reference's own kernels).
#include "fsr_compat.h"

extern "C" {

void w_bindTextures(uint* edge, int* tri, uint* nverts, uint* edge_corners)
{
    bindTextures(edge, tri, nverts, edge_corners);
}

void w_launchSpatialGridBuilding(const ParticleArray* p, const ScalarFieldGrid* d, uint n,
                                 const ParticleIndexRangeGrid* r, const DensityGrid* f, const GridInfo* gi)
{
    launchSpatialGridBuilding(*p, *d, n, *r, *f, *gi);
}

void w_launchExtractionOfSurfaceParticles(const dim3* g, const dim3* b, const SimParam* s, const DensityGrid* f,
                                          const IsSurfaceGrid* sf, const ParticleIndexRangeGrid* r)
{
    launchExtractionOfSurfaceParticles(*g, *b, *s, *f, *sf, *r);
}

void w_launchExtractionOfSurfaceAndInvolveParticles(const dim3* g, const dim3* b, const SimParam* s,
                                                    const DensityGrid* f, const NumInvolveParticlesGrid* ni,
                                                    const IsSurfaceGrid* sf, const ParticleIndexRangeGrid* r)
{
    launchExtractionOfSurfaceAndInvolveParticles(*g, *b, *s, *f, *ni, *sf, *r);
}

void w_launchExtractionOfSurfaceParticlesForAkinci(const dim3* g, const dim3* b, const SimParam* s,
                                                   const ParticleArray* p, const ScalarFieldGrid* d,
                                                   const ParticleIndexRangeGrid* r, const GridInfo* gi,
                                                   const IsSurfaceGrid* sf)
{
    launchExtractionOfSurfaceParticlesForAkinci(*g, *b, *s, *p, *d, *r, *gi, *sf);
}

void w_launchEstimationOfSurfaceVertices(const dim3* g, const dim3* b, const SimParam* s, const GridInfo* sci,
                                         const ParticleArray* p, const IsSurfaceGrid* sf,
                                         const ParticleIndexRangeGrid* r, const IsSurfaceGrid* band)
{
    launchEstimationOfSurfaceVertices(*g, *b, *s, *sci, *p, *sf, *r, *band);
}

uint w_launchThrustExclusivePrefixSumScan(uint* out, uint* in, uint n)
{
    return launchThrustExclusivePrefixSumScan(out, in, n);
}

void w_launchCompactSurfaceVertex(const dim3* g, const dim3* b, const SurfaceVerticesIndexArray* sv,
                                  const IsSurfaceGrid* scan, const IsSurfaceGrid* band, const SimParam* s)
{
    launchCompactSurfaceVertex(*g, *b, *sv, *scan, *band, *s);
}

void w_launchUpdateScalarGridValuesCompacted(const dim3* g, const dim3* b, const SurfaceVerticesIndexArray* sv,
                                             uint nsv, const ParticleIndexRangeGrid* r, const ParticleArray* p,
                                             const ScalarFieldGrid* f, const GridInfo* spi, const GridInfo* sci,
                                             const SimParam* s)
{
    launchUpdateScalarGridValuesCompacted(*g, *b, *sv, nsv, *r, *p, *f, *spi, *sci, *s);
}

void w_launchDetectValidSurfaceCubes(const dim3* g, const dim3* b, const SurfaceVerticesIndexArray* sv, uint nsv,
                                     const ScalarFieldGrid* f, const IsValidSurfaceGrid* v, const NumVerticesGrid* nv,
                                     const IsSurfaceGrid* band, const SimParam* s)
{
    launchDetectValidSurfaceCubes(*g, *b, *sv, nsv, *f, *v, *nv, *band, *s);
}

void w_launchDetectionOfValidSurfaceCubesForAkinci(const dim3* g, const dim3* b, const SurfaceVerticesIndexArray* sv,
                                                   uint nsv, const ScalarFieldGrid* f, const IsValidSurfaceGrid* v,
                                                   const IsSurfaceGrid* band, const SimParam* s)
{
    launchDetectionOfValidSurfaceCubesForAkinci(*g, *b, *sv, nsv, *f, *v, *band, *s);
}

void w_launchCompactValidSurfaceCubes(const dim3* g, const dim3* b, const ValidSurfaceIndexArray* idx,
                                      const IsValidSurfaceGrid* scan, const IsValidSurfaceGrid* v, const SimParam* s)
{
    launchCompactValidSurfaceCubes(*g, *b, *idx, *scan, *v, *s);
}

void w_launchGenerateTriangles(const dim3* g, const dim3* b, const SurfaceVerticesIndexArray* sv,
                               const ValidSurfaceIndexArray* vi, const GridInfo* sci, const NumVerticesGrid* nvs,
                               const ScalarFieldGrid* f, const Float3Grid* pos, const Float3Grid* nrm,
                               const SimParam* s)
{
    launchGenerateTriangles(*g, *b, *sv, *vi, *sci, *nvs, *f, *pos, *nrm, *s);
}

void w_launchCalculationOfMeanAndSmoothParticles(const dim3* g, const dim3* b, const SimParam* s,
                                                 const ParticleArray* p, const ParticleArray* m,
                                                 const ParticleArray* sm, const ParticleIndexRangeGrid* r,
                                                 const GridInfo* spi)
{
    launchCalculationOfMeanAndSmoothParticles(*g, *b, *s, *p, *m, *sm, *r, *spi);
}

void w_launchCompactationOfSurfaceVerticesAndParticles(const dim3* g, const dim3* b, const SimParam* s,
                                                       const IsSurfaceGrid* band, const IsSurfaceGrid* bscan,
                                                       const NumInvolveParticlesGrid* ni,
                                                       const NumInvolveParticlesGrid* niscan,
                                                       const ParticleIndexRangeGrid* r,
                                                       const SurfaceVerticesIndexArray* sv,
                                                       const SurfaceParticlesIndexArray* sp)
{
    launchCompactationOfSurfaceVerticesAndParticles(*g, *b, *s, *band, *bscan, *ni, *niscan, *r, *sv, *sp);
}

void w_launchCalculationOfTransformMatricesForParticles(const dim3* g, const dim3* b, const SimParam* s,
                                                        const GridInfo* spi, const ParticleArray* m,
                                                        const ParticleArray* p, const ParticleIndexRangeGrid* r,
                                                        const SurfaceParticlesIndexArray* idx,
                                                        const MatrixArray* mats)
{
    launchCalculationOfTransformMatricesForParticles(*g, *b, *s, *spi, *m, *p, *r, *idx, *mats);
}

void w_launchComputationOfScalarFieldGrid(const dim3* g, const dim3* b, const SimParam* s, uint nsv,
                                          const GridInfo* sci, const GridInfo* spi, const MatrixArray* mats,
                                          const ParticleArray* sm, const ScalarFieldGrid* d,
                                          const ParticleIndexRangeGrid* r, const SurfaceVerticesIndexArray* sv,
                                          const NumInvolveParticlesGrid* ni, const NumInvolveParticlesGrid* niscan,
                                          const ScalarFieldGrid* f)
{
    launchComputationOfScalarFieldGrid(*g, *b, *s, nsv, *sci, *spi, *mats, *sm, *d, *r, *sv, *ni, *niscan, *f);
}

}  // extern "C"
