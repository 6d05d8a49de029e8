/*
 * fsr_compat.h - the reference's kernel-level C ABI, implemented by
 * libfsr_gb300.so on the GB300.
 *
 * Same symbol names, parameter lists and struct layouts as the extern "C"
 * launchers declared in FluidSurfaceReconstruction/GPU/ReconstructionCUDA.cuh
 * (lines 17-248), so the reference's host classes (ReconstructorGPU*.cpp)
 * link against this library unchanged.  Semantics follow each reference
 * kernel on the reference's dense buffers; the GPU work is this library's
 * own kernels.  Differences, all documented per function below:
 *  - the grid/block arguments only define the logical thread domain
 *    (gridDim.x*gridDim.y*gridDim.z * blockDim.x*blockDim.y*blockDim.z
 *    threads, linearised as getThreadIdGlobal does, cu:40-47); the kernels
 *    run with their own launch shapes;
 *  - the smoothing launcher runs exactly particleArray.size threads (the
 *    reference's bound "threadId > size" lets thread `size` read and write
 *    one element past the arrays, cu:609);
 *  - particles outside the grid are skipped by launchSpatialGridBuilding
 *    (the reference writes out of bounds, cu:1391-1395);
 *  - errors are reported through cudaGetLastError (launchers are void, as in
 *    the reference) instead of exiting the process.
 * launchUpdateScalarGridValues (cuh:45-55) is not provided: the reference
 * declares it but never defines it.
 *
 * C++ only (Grid<T> is a template).  Define FSR_COMPAT_NO_TYPES when the
 * reference's own Defines.h already provides the types.
 */
#ifndef FSR_COMPAT_H
#define FSR_COMPAT_H

#include <cuda_runtime.h>
#include <vector_types.h>

#ifndef FSR_COMPAT_NO_TYPES
typedef unsigned int uint;

/* Defines.h:18-32 */
struct SimParam {
    float particleRadius;
    float particleMass;
    float smoothingRadius;
    float smoothingRadiusSq;
    float smoothingRadiusInv;
    float lambdaForSmoothed;
    float anisotropicRadius;
    float isoValue;
    uint scSpGridResRatio;
    uint expandExtent;
    uint minNumNeighbors;
    float spatialCellSizeScale;
};

/* Defines.h:35-42: non-owning view of a device array / grid */
template <typename T>
struct Grid {
    T* grid;
    unsigned long long size;
    unsigned long long count;
    uint3 resolution;
};

struct IndexRange { uint start, end; };                 /* Defines.h:45 */
struct ParticlePosition { float3 pos; };                /* Defines.h:48 */
struct ScalarValue { float value; };                    /* Defines.h:51 */
struct MatrixValue {                                    /* Defines.h:54-59 */
    float a11, a12, a13;
    float a21, a22, a23;
    float a31, a32, a33;
};
struct GridInfo {                                       /* Defines.h:62-68 */
    float3 minPos;
    float3 maxPos;
    float cellSize;
    uint3 resolution;
};

typedef Grid<uint> UintGrid;
typedef Grid<float> FloatGrid;
typedef Grid<float3> Float3Grid;
typedef Grid<float> DensityGrid;
typedef Grid<ParticlePosition> ParticleArray;
typedef Grid<IndexRange> ParticleIndexRangeGrid;
typedef Grid<ScalarValue> ScalarFieldGrid;
typedef Grid<uint> IsSurfaceGrid;
typedef Grid<uint> NumInvolveParticlesGrid;
typedef Grid<uint> NumVerticesGrid;
typedef Grid<uint> IsValidSurfaceGrid;
typedef Grid<uint> SurfaceParticlesIndexArray;
typedef Grid<uint> SurfaceVerticesIndexArray;
typedef Grid<uint> ValidSurfaceIndexArray;
typedef Grid<MatrixValue> MatrixArray;
#endif

/* cuh:17-22.  Records the caller's marching-cubes tables; the kernels use
 * this library's constant-memory copy of the same tables. */
extern "C" void bindTextures(uint* d_edgeTable, int* d_edgeIndicesOfTriangleTable, uint* d_numVerticesTable,
                             uint* d_vertexIndicesOfEdgeTable);

/* cuh:25-32 (cu:70-120): flag-grid surface particles. */
extern "C" void launchExtractionOfSurfaceParticles(dim3 gridDim_, dim3 blockDim_, SimParam simParam,
                                                   DensityGrid flagGrid, IsSurfaceGrid surfaceParticlesFlagGrid,
                                                   ParticleIndexRangeGrid particleIndexRangeGrid);

/* cuh:35-42 (cu:123-175): band from the occupancy grid's 0.5 crossings
 * (no caller in the reference). */
extern "C" void launchEstimateSurfaceVertices(dim3 gridDim, dim3 blockDim, DensityGrid densityGrid,
                                              IsSurfaceGrid isSurfaceGrid, uint scSearchExt, SimParam params);

/* cuh:58-65 (cu:293-304) */
extern "C" void launchCompactSurfaceVertex(dim3 gridDim_, dim3 blockDim_, SurfaceVerticesIndexArray svIndexArray,
                                           IsSurfaceGrid isSurfaceGridScan, IsSurfaceGrid isSurfaceGrid,
                                           SimParam params);

/* cuh:68-79 (cu:230-289, 308-324): ZB05 field at the band vertices. */
extern "C" void launchUpdateScalarGridValuesCompacted(dim3 gridDim_, dim3 blockDim_,
                                                      SurfaceVerticesIndexArray svIndexArray, uint numSurfaceVertices,
                                                      ParticleIndexRangeGrid particleIndexRangeGrid,
                                                      ParticleArray particleArray, ScalarFieldGrid ScalarFieldGrid,
                                                      GridInfo spatialGridInfo, GridInfo scalarGridInfo,
                                                      SimParam params);

/* cuh:82-92 (cu:328-364) */
extern "C" void launchDetectValidSurfaceCubes(dim3 gridDim_, dim3 blockDim_, SurfaceVerticesIndexArray svIndexArray,
                                              uint numSurfaceVertices, ScalarFieldGrid vGrid,
                                              IsValidSurfaceGrid isValidSurfaceGrid, NumVerticesGrid numVerticesGrid,
                                              IsSurfaceGrid isSfGrid, SimParam params);

/* cuh:95-102 (cu:367-380) */
extern "C" void launchCompactValidSurfaceCubes(dim3 gridDim_, dim3 blockDim_, ValidSurfaceIndexArray indexArray,
                                               IsValidSurfaceGrid validSurfaceGridScan,
                                               IsValidSurfaceGrid validSurafceGrid, SimParam params);

/* cuh:105-116 (cu:383-463) */
extern "C" void launchGenerateTriangles(dim3 gridDim_, dim3 blockDim_, SurfaceVerticesIndexArray surfaceIndexInGridArray,
                                        ValidSurfaceIndexArray validIndexInSurfaceArray, GridInfo scGridInfo,
                                        NumVerticesGrid numVerticesGridScan, ScalarFieldGrid ScalarFieldGrid,
                                        Float3Grid posGrid, Float3Grid norGrid, SimParam params);

/* cuh:118-119 (cu:1154-1172): exclusive scan, returns the total (last
 * input + last output, read back to the host as the reference does). */
extern "C" uint launchThrustExclusivePrefixSumScan(uint* output, uint* input, uint numElements);

/* cuh:134-142 (cu:466-551) */
extern "C" void launchExtractionOfSurfaceAndInvolveParticles(dim3 gridDim_, dim3 blockDim_, SimParam simParam,
                                                             DensityGrid flagGrid,
                                                             NumInvolveParticlesGrid numInvolveParticlesGrid,
                                                             IsSurfaceGrid surfaceParticlesFlagGrid,
                                                             ParticleIndexRangeGrid particleIndexRangeGrid);

/* cuh:145-154 (cu:554-595) */
extern "C" void launchEstimationOfSurfaceVertices(dim3 gridDim_, dim3 blockDim_, SimParam simParam,
                                                  GridInfo scalarGridInfo, ParticleArray particleArray,
                                                  IsSurfaceGrid surfaceParticlesFlagGrid,
                                                  ParticleIndexRangeGrid particleIndexRangeGrid,
                                                  IsSurfaceGrid isSurfaceGrid);

/* cuh:157-166 (cu:598-658) */
extern "C" void launchCalculationOfMeanAndSmoothParticles(dim3 gridDim_, dim3 blockDim_, SimParam simParam,
                                                          ParticleArray particleArray, ParticleArray meanParticleArray,
                                                          ParticleArray smoothedParticleArray,
                                                          ParticleIndexRangeGrid particleIndexRangeGrid,
                                                          GridInfo spatialGridInfo);

/* cuh:169-180 (cu:661-686) */
extern "C" void launchCompactationOfSurfaceVerticesAndParticles(
    dim3 gridDim_, dim3 blockDim_, SimParam simParam, IsSurfaceGrid isSurfaceGrid, IsSurfaceGrid isSurfaceGridScan,
    NumInvolveParticlesGrid numInvolveParticlesGrid, NumInvolveParticlesGrid numInvolveParticlesGridScan,
    ParticleIndexRangeGrid particleIndexRangeGrid, SurfaceVerticesIndexArray surfaceVerticesIndexArray,
    SurfaceParticlesIndexArray surfaceParticlesIndexArray);

/* cuh:183-193 (cu:689-827): G per involved particle (this library's
 * eigen-solver in place of GPU/SVD3.cuh). */
extern "C" void launchCalculationOfTransformMatricesForParticles(
    dim3 gridDim_, dim3 blockDim_, SimParam simParam, GridInfo spatialGridInfo, ParticleArray meanParticleArray,
    ParticleArray particleArray, ParticleIndexRangeGrid particleIndexRangeGrid,
    SurfaceParticlesIndexArray surfaceParticlesIndexArray, MatrixArray svdMatricesArray);

/* cuh:196-211 (cu:830-906) */
extern "C" void launchComputationOfScalarFieldGrid(
    dim3 gridDim_, dim3 blockDim_, SimParam simParam, uint numSurfaceVertices, GridInfo scalarGridInfo,
    GridInfo spatialGridInfo, MatrixArray svdMatricesArray, ParticleArray smoothedParticleArray,
    ScalarFieldGrid particlesDensityArray, ParticleIndexRangeGrid particleIndexRangeGrid,
    SurfaceVerticesIndexArray surfaceVerticesIndexArray, NumInvolveParticlesGrid numInvolveParticlesGrid,
    NumInvolveParticlesGrid numInvolveParticlesGridScan, ScalarFieldGrid ScalarFieldGrid);

/* cuh:216-225 (cu:909-971) */
extern "C" void launchExtractionOfSurfaceParticlesForAkinci(dim3 gridDim_, dim3 blockDim_, SimParam simParam,
                                                            ParticleArray particlesArray,
                                                            ScalarFieldGrid particlesDensityArray,
                                                            ParticleIndexRangeGrid particleIndexRangeGrid,
                                                            GridInfo spatialGridInfo,
                                                            IsSurfaceGrid surfaceParticlesFlagGrid);

/* cuh:228-237 (cu:974-1008) */
extern "C" void launchDetectionOfValidSurfaceCubesForAkinci(dim3 gridDim_, dim3 blockDim_,
                                                            SurfaceVerticesIndexArray svIndexArray,
                                                            uint numSurfaceVertices, ScalarFieldGrid vGrid,
                                                            IsValidSurfaceGrid isValidSurfaceGrid,
                                                            IsSurfaceGrid isSfGrid, SimParam params);

/* cuh:241-248 (cu:1437-1481): hash, stable in-place sort of positions and
 * densities by cell, cell ranges, occupancy grid. */
extern "C" void launchSpatialGridBuilding(ParticleArray particlesArray, ScalarFieldGrid densitiesArray,
                                          uint numParticles, ParticleIndexRangeGrid particlesIndexRangerArray,
                                          DensityGrid densityGrid, GridInfo spatialGridInfo);

#endif
