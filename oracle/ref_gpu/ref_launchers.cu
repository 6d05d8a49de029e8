// The reference's kernel-level C ABI (the launch* functions declared in
// GPU/ReconstructionCUDA.cuh:17-248), implemented by launching the
// reference's OWN kernels: the device code of ReconstructionCUDA.cu built
// for sm_103a by oracle/ref_gpu/build_ref_gpu.sh into
// oracle/_ref/ref_kernels_sm103a.cubin, loaded here with the driver API.
// TEST AND MEASUREMENT INFRASTRUCTURE: the GPU baseline of bench.py and
// tests/test_gpu_reference_build.py; nothing of the product links it.
//
// Each launcher does what the reference's does (ReconstructionCUDA.cu:
// 1010-1481): it launches one kernel with the caller's grid and block on the
// legacy default stream and synchronises the device; the two thrust calls
// (sort_by_key of the hashed particles, cu:1463-1466, and the exclusive
// scans with their two 4-byte read-backs, cu:1154-1172) are the same thrust
// calls; launchSpatialGridBuilding allocates and frees its hash array per
// call (cu:1446-1480).  Kernels are found by their mangled names, which
// begin with "_Z" followed by the length and the kernel's name (the
// reference's kernels are free functions without overloads).
//
// The marching-cubes tables: bindTextures stores the caller's table
// pointers in the module's table-pointer globals (the recipe turned the four
// textures into __device__ pointers).
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/scan.h>
#include <thrust/sort.h>
#include <thrust/tuple.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fsr_compat.h"

namespace {

std::mutex g_mu;
CUmodule g_mod = nullptr;
std::map<std::string, CUfunction> g_fn;
std::string g_err;

const char* module_path()
{
    const char* p = getenv("FSR_REF_CUBIN");
    return p ? p : "";
}

bool load_module()
{
    if (g_mod) return true;
    cudaFree(0);  // the runtime's primary context becomes current
    CUresult r = cuModuleLoad(&g_mod, module_path());
    if (r != CUDA_SUCCESS) {
        g_err = std::string("cuModuleLoad failed for ") + module_path();
        g_mod = nullptr;
        return false;
    }
    unsigned count = 0;
    cuModuleGetFunctionCount(&count, g_mod);
    std::vector<CUfunction> fs(count);
    cuModuleEnumerateFunctions(fs.data(), count, g_mod);
    for (CUfunction f : fs) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name) g_fn[name] = f;
    }
    return true;
}

CUfunction kernel(const char* base)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!load_module()) return nullptr;
    const std::string prefix = "_Z" + std::to_string(strlen(base)) + base;
    for (auto& kv : g_fn)
        if (kv.first.compare(0, prefix.size(), prefix) == 0) return kv.second;
    g_err = std::string("kernel not in module: ") + base;
    return nullptr;
}

template <class... A>
void launch(const char* name, dim3 g, dim3 b, unsigned smem, A&... args)
{
    CUfunction f = kernel(name);
    if (!f) return;
    void* params[] = {(void*)&args...};
    if (cuLaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, smem, nullptr, params, nullptr) != CUDA_SUCCESS)
        g_err = std::string("launch failed: ") + name;
}

}  // namespace

extern "C" const char* ref_gpu_last_error() { return g_err.c_str(); }

extern "C" int ref_gpu_load(const char* cubin_path)
{
    if (cubin_path) setenv("FSR_REF_CUBIN", cubin_path, 1);
    std::lock_guard<std::mutex> lock(g_mu);
    return load_module() ? 0 : 1;
}

extern "C" void bindTextures(uint* d_edgeTable, int* d_edgeIndicesOfTriangleTable, uint* d_numVerticesTable,
                             uint* d_vertexIndicesOfEdgeTable)
{
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!load_module()) return;
    }
    const char* names[4] = {"edgeTex", "edgeIndexesOfTriangleTex", "numVerticesTex", "vertexIndexesOfEdgeTex"};
    const void* ptrs[4] = {d_edgeTable, d_edgeIndicesOfTriangleTable, d_numVerticesTable, d_vertexIndicesOfEdgeTable};
    for (int i = 0; i < 4; ++i) {
        CUdeviceptr sym = 0;
        size_t bytes = 0;
        if (cuModuleGetGlobal(&sym, &bytes, g_mod, names[i]) != CUDA_SUCCESS || bytes != sizeof(void*)) {
            g_err = std::string("table pointer not in module: ") + names[i];
            return;
        }
        cuMemcpyHtoD(sym, &ptrs[i], sizeof(void*));
    }
}

extern "C" void launchExtractionOfSurfaceParticles(dim3 g, dim3 b, SimParam simParam, DensityGrid flagGrid,
                                                   IsSurfaceGrid surfaceParticlesFlagGrid,
                                                   ParticleIndexRangeGrid particleIndexRangeGrid)
{
    launch("extractionOfSurfaceParticles", g, b, 0, simParam, flagGrid, surfaceParticlesFlagGrid,
           particleIndexRangeGrid);
    cudaDeviceSynchronize();
}

extern "C" void launchCompactSurfaceVertex(dim3 g, dim3 b, SurfaceVerticesIndexArray svIndexArray,
                                           IsSurfaceGrid isSurfaceGridScan, IsSurfaceGrid isSurfaceGrid,
                                           SimParam params)
{
    launch("compactSurfaceVertex", g, b, 0, svIndexArray, isSurfaceGridScan, isSurfaceGrid, params);
    cudaDeviceSynchronize();
}

extern "C" void launchUpdateScalarGridValuesCompacted(dim3 g, dim3 b, SurfaceVerticesIndexArray svIndexArray,
                                                      uint numSurfaceVertices,
                                                      ParticleIndexRangeGrid particleIndexRangeGrid,
                                                      ParticleArray particleArray, ScalarFieldGrid scalarFieldGrid,
                                                      GridInfo spatialGridInfo, GridInfo scalarGridInfo,
                                                      SimParam params)
{
    launch("updateScalarGridValuesCompacted", g, b, 0, svIndexArray, numSurfaceVertices, particleIndexRangeGrid,
           particleArray, scalarFieldGrid, spatialGridInfo, scalarGridInfo, params);
    cudaDeviceSynchronize();
}

extern "C" void launchDetectValidSurfaceCubes(dim3 g, dim3 b, SurfaceVerticesIndexArray svIndexArray,
                                              uint numSurfaceVertices, ScalarFieldGrid vGrid,
                                              IsValidSurfaceGrid isValidSurfaceGrid, NumVerticesGrid numVerticesGrid,
                                              IsSurfaceGrid isSfGrid, SimParam params)
{
    launch("detectValidSurfaceCubes", g, b, 0, svIndexArray, numSurfaceVertices, vGrid, isValidSurfaceGrid,
           numVerticesGrid, isSfGrid, params);
    cudaDeviceSynchronize();
}

extern "C" void launchCompactValidSurfaceCubes(dim3 g, dim3 b, ValidSurfaceIndexArray indexArray,
                                               IsValidSurfaceGrid validSurfaceGridScan,
                                               IsValidSurfaceGrid validSurafceGrid, SimParam params)
{
    launch("compactValidSurfaceCubes", g, b, 0, indexArray, validSurfaceGridScan, validSurafceGrid, params);
    cudaDeviceSynchronize();
}

extern "C" void launchGenerateTriangles(dim3 g, dim3 b, SurfaceVerticesIndexArray surfaceIndexInGridArray,
                                        ValidSurfaceIndexArray validIndexInSurfaceArray, GridInfo scGridInfo,
                                        NumVerticesGrid numVerticesGridScan, ScalarFieldGrid scalarFieldGrid,
                                        Float3Grid posGrid, Float3Grid norGrid, SimParam params)
{
    launch("generateTriangles", g, b, 0, surfaceIndexInGridArray, validIndexInSurfaceArray, scGridInfo,
           numVerticesGridScan, scalarFieldGrid, posGrid, norGrid, params);
    cudaDeviceSynchronize();
}

extern "C" uint launchThrustExclusivePrefixSumScan(uint* output, uint* input, uint numElements)
{
    thrust::exclusive_scan(thrust::device_ptr<uint>(input), thrust::device_ptr<uint>(input + numElements),
                           thrust::device_ptr<uint>(output));
    cudaDeviceSynchronize();
    uint last = 0, last_scan = 0;
    cudaMemcpy(&last, input + numElements - 1, sizeof(uint), cudaMemcpyDeviceToHost);
    cudaMemcpy(&last_scan, output + numElements - 1, sizeof(uint), cudaMemcpyDeviceToHost);
    return last + last_scan;
}

extern "C" void launchExtractionOfSurfaceAndInvolveParticles(dim3 g, dim3 b, SimParam simParam,
                                                             DensityGrid flagGrid,
                                                             NumInvolveParticlesGrid numInvolveParticlesGrid,
                                                             IsSurfaceGrid surfaceParticlesFlagGrid,
                                                             ParticleIndexRangeGrid particleIndexRangeGrid)
{
    launch("extractionOfSurfaceAndInvolveParticles", g, b, 0, simParam, flagGrid, numInvolveParticlesGrid,
           surfaceParticlesFlagGrid, particleIndexRangeGrid);
    cudaDeviceSynchronize();
}

extern "C" void launchEstimationOfSurfaceVertices(dim3 g, dim3 b, SimParam simParam, GridInfo scalarGridInfo,
                                                  ParticleArray particleArray, IsSurfaceGrid surfaceParticlesFlagGrid,
                                                  ParticleIndexRangeGrid particleIndexRangeGrid,
                                                  IsSurfaceGrid isSurfaceGrid)
{
    launch("estimationOfSurfaceVertices", g, b, 0, simParam, scalarGridInfo, particleArray, surfaceParticlesFlagGrid,
           particleIndexRangeGrid, isSurfaceGrid);
    cudaDeviceSynchronize();
}

extern "C" void launchCalculationOfMeanAndSmoothParticles(dim3 g, dim3 b, SimParam simParam,
                                                          ParticleArray particleArray, ParticleArray meanParticleArray,
                                                          ParticleArray smoothedParticleArray,
                                                          ParticleIndexRangeGrid particleIndexRangeGrid,
                                                          GridInfo spatialGridInfo)
{
    launch("calculationOfMeanAndSmoothParticles", g, b, 0, simParam, particleArray, meanParticleArray,
           smoothedParticleArray, particleIndexRangeGrid, spatialGridInfo);
    cudaDeviceSynchronize();
}

extern "C" void launchCompactationOfSurfaceVerticesAndParticles(
    dim3 g, dim3 b, SimParam simParam, IsSurfaceGrid isSurfaceGrid, IsSurfaceGrid isSurfaceGridScan,
    NumInvolveParticlesGrid numInvolveParticlesGrid, NumInvolveParticlesGrid numInvolveParticlesGridScan,
    ParticleIndexRangeGrid particleIndexRangeGrid, SurfaceVerticesIndexArray surfaceVerticesIndexArray,
    SurfaceParticlesIndexArray surfaceParticlesIndexArray)
{
    launch("compactationOfSurfaceVerticesAndParticles", g, b, 0, simParam, isSurfaceGrid, isSurfaceGridScan,
           numInvolveParticlesGrid, numInvolveParticlesGridScan, particleIndexRangeGrid, surfaceVerticesIndexArray,
           surfaceParticlesIndexArray);
    cudaDeviceSynchronize();
}

extern "C" void launchCalculationOfTransformMatricesForParticles(
    dim3 g, dim3 b, SimParam simParam, GridInfo spatialGridInfo, ParticleArray meanParticleArray,
    ParticleArray particleArray, ParticleIndexRangeGrid particleIndexRangeGrid,
    SurfaceParticlesIndexArray surfaceParticlesIndexArray, MatrixArray svdMatricesArray)
{
    launch("calculationOfTransformMatricesForParticles", g, b, 0, simParam, spatialGridInfo, meanParticleArray,
           particleArray, particleIndexRangeGrid, surfaceParticlesIndexArray, svdMatricesArray);
    cudaDeviceSynchronize();
}

extern "C" void launchComputationOfScalarFieldGrid(
    dim3 g, dim3 b, SimParam simParam, uint numSurfaceVertices, GridInfo scalarGridInfo, GridInfo spatialGridInfo,
    MatrixArray svdMatricesArray, ParticleArray smoothedParticleArray, ScalarFieldGrid particlesDensityArray,
    ParticleIndexRangeGrid particleIndexRangeGrid, SurfaceVerticesIndexArray surfaceVerticesIndexArray,
    NumInvolveParticlesGrid numInvolveParticlesGrid, NumInvolveParticlesGrid numInvolveParticlesGridScan,
    ScalarFieldGrid scalarFieldGrid)
{
    launch("computationOfScalarFieldGrid", g, b, 0, simParam, numSurfaceVertices, scalarGridInfo, spatialGridInfo,
           svdMatricesArray, smoothedParticleArray, particlesDensityArray, particleIndexRangeGrid,
           surfaceVerticesIndexArray, numInvolveParticlesGrid, numInvolveParticlesGridScan, scalarFieldGrid);
    cudaDeviceSynchronize();
}

extern "C" void launchExtractionOfSurfaceParticlesForAkinci(dim3 g, dim3 b, SimParam simParam,
                                                            ParticleArray particlesArray,
                                                            ScalarFieldGrid particlesDensityArray,
                                                            ParticleIndexRangeGrid particleIndexRangeGrid,
                                                            GridInfo spatialGridInfo,
                                                            IsSurfaceGrid surfaceParticlesFlagGrid)
{
    launch("extractionOfSurfaceParticlesUsingColorField", g, b, 0, simParam, particlesArray, particlesDensityArray,
           particleIndexRangeGrid, spatialGridInfo, surfaceParticlesFlagGrid);
    cudaDeviceSynchronize();
}

extern "C" void launchDetectionOfValidSurfaceCubesForAkinci(dim3 g, dim3 b, SurfaceVerticesIndexArray svIndexArray,
                                                            uint numSurfaceVertices, ScalarFieldGrid vGrid,
                                                            IsValidSurfaceGrid isValidSurfaceGrid,
                                                            IsSurfaceGrid isSfGrid, SimParam params)
{
    launch("detectionOfValidSurfaceCubesForAkinci", g, b, 0, svIndexArray, numSurfaceVertices, vGrid,
           isValidSurfaceGrid, isSfGrid, params);
    cudaDeviceSynchronize();
}

extern "C" void launchSpatialGridBuilding(ParticleArray particlesArray, ScalarFieldGrid densitiesArray,
                                          uint numParticles, ParticleIndexRangeGrid particlesIndexRangerArray,
                                          DensityGrid flagGrid, GridInfo spatialGridInfo)
{
    uint* hash = nullptr;
    cudaMalloc((void**)&hash, numParticles * sizeof(uint));
    const unsigned threads = 256;
    const unsigned blocks = (numParticles + threads - 1) / threads;
    launch("calcParticlesHashKernel", dim3(blocks), dim3(threads), 0, hash, particlesArray, numParticles, flagGrid,
           spatialGridInfo);
    cudaDeviceSynchronize();
    thrust::device_ptr<ParticlePosition> pos(particlesArray.grid);
    thrust::device_ptr<ScalarValue> den(densitiesArray.grid);
    thrust::sort_by_key(thrust::device_ptr<uint>(hash), thrust::device_ptr<uint>(hash + numParticles),
                        thrust::make_zip_iterator(thrust::make_tuple(pos, den)));
    cudaDeviceSynchronize();
    cudaMemset(particlesIndexRangerArray.grid, 0xff, particlesIndexRangerArray.size * sizeof(IndexRange));
    launch("findCellRangeKernel", dim3(blocks), dim3(threads), (threads + 1) * sizeof(uint),
           particlesIndexRangerArray, numParticles, hash);
    cudaDeviceSynchronize();
    cudaFree(hash);
}
