/*
 * Stage-level C API shared by the CPU oracle (fsr_oracle.c) and by the
 * host-compiled reference kernels (ref_driver.cpp).  TEST INFRASTRUCTURE:
 * only tests, the smoke check and the benchmark's CPU-baseline leg load the
 * libraries that implement it.
 *
 * Every stage mirrors one launch of the reference's per-frame pipeline
 * (FluidSurfaceReconstruction/GPU/ReconstructorGPUOurs*.cpp, *Akinci12.cpp)
 * and works on the reference's dense layouts:
 *   pos      N x float3 (ParticlePosition, Defines.h:48), sorted order
 *   ranges   C x {start,end} u32 (IndexRange, Defines.h:45), 0xFFFFFFFF = empty
 *   flag     C x f32 occupancy (1.0 = occupied), the reference's "flag grid"
 *   sflag    N x u32 surface-particle flags
 *   isSurf   V x u32 narrow-band flags on the scalar grid
 *   phi      V x real_t dense scalar field (caller pre-fills it)
 * real_t is float in the FP32 builds and double in the FP64 oracle build.
 * Every function returns 0 on success and a negative code on bad input.
 */
#ifndef FSR_STAGE_API_H
#define FSR_STAGE_API_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field order and size (48 B) as SimParam, Defines.h:18-32. */
typedef struct o_simparam {
    float particleRadius, particleMass, smoothingRadius, smoothingRadiusSq;
    float smoothingRadiusInv, lambdaForSmoothed, anisotropicRadius, isoValue;
    uint32_t scSpGridResRatio, expandExtent, minNumNeighbors;
    float spatialCellSizeScale;
} o_simparam;

/* Same field order and size (40 B) as GridInfo, Defines.h:62-68. */
typedef struct o_gridinfo {
    float minPos[3];
    float maxPos[3];
    float cellSize;
    uint32_t res[3];
} o_gridinfo;

#ifdef __cplusplus
}
#endif
#endif
