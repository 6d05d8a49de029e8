/*
 * fsr_reconstructor.hpp - the reference's file-driven reconstructor classes
 * over the fsr_* C ABI (header only; link with libfsr_gb300.so).
 *
 * Public surface of ReconstructorGPU (FluidSurfaceReconstruction/GPU/
 * ReconstructorGPU.h:14-30) and its subclasses (ReconstructorGPUOursZB05.h,
 * ReconstructorGPUOursYu13.h, ReconstructorGPUAkinci12.h): the constructor
 * (directory, file pattern, frames [from, to)), reconstruct(),
 * getAlgorithmType(), setOutputMeshFile / setOutputConfigFile /
 * setOutputVisualizeFile, getSimulationParameters(), getNumberOfParticles()
 * and getTimeConsumingSequence().  reconstruct() follows
 * ReconstructorGPU::reconstruct (ReconstructorGPU.cpp:25-79): each frame's
 * <directory><pattern % frame>.xyz is read, uploaded outside the timer,
 * reconstructed (timed: hashing to mesh), written as .obj when enabled;
 * afterwards "<algorithm type>.time" gets one line of per-frame
 * milliseconds (appended, as ReconstructorGPU.cpp:306-337 does) and, with
 * the config output on, "<algorithm type>.config" the averages of
 * ReconstructorGPU.cpp:339-395 (triangles, surface-particle ratio,
 * surface-vertex ratio, then four stage-time sums in milliseconds).
 *
 * setOutputVisualizeFile writes each frame's .vis dump (fsr_write_vis).
 *
 * Differences: errors throw fsr_gb300::Error instead of printing and exiting
 * the process.  Extensions: setBinarySidecar (.xyzb) and setIndexedMesh
 * (welded .obj).
 */
#ifndef FSR_RECONSTRUCTOR_HPP
#define FSR_RECONSTRUCTOR_HPP

#include <cstdio>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "fsr.h"
#include "fsr_compat.h"

namespace fsr_gb300 {

class Error : public std::runtime_error {
public:
    Error(fsr_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    fsr_status status;
};

class ReconstructorGPU {
public:
    typedef std::shared_ptr<ReconstructorGPU> ptr;

    ReconstructorGPU(const std::string& directory, const std::string& filePattern, unsigned int from,
                     unsigned int to, uint32_t method, int device = 0)
        : mDirectory(directory), mPattern(filePattern), mFrom(from), mTo(to), mDevice(device)
    {
        fsr_default_params(method, &mParams);
        mParams.flags |= FSR_FLAG_STAGE_TIMING;
    }
    virtual ~ReconstructorGPU()
    {
        if (mHandle) fsr_destroy(mHandle);
    }
    ReconstructorGPU(const ReconstructorGPU&) = delete;
    ReconstructorGPU& operator=(const ReconstructorGPU&) = delete;

    virtual std::string getAlgorithmType() = 0;

    virtual void reconstruct()
    {
        if (mFrom >= mTo) return;  // "Wrong settings occur for frame range."
        if (!mHandle) check(fsr_create(&mParams, mDevice, &mHandle), "fsr_create");
        mTimeConsuming.clear();
        std::vector<double> tri, spr, svr, es, sf, mc;
        for (unsigned int f = mFrom; f < mTo; ++f) {
            double ms = 0.0;
            const uint32_t flags = (mSaveObjFile ? FSR_FILES_WRITE_OBJ : 0u) | (mSidecar ? FSR_FILES_SIDECAR : 0u) |
                                   (mIndexed ? FSR_FILES_INDEXED_OBJ : 0u) | (mSaveVisFile ? FSR_FILES_WRITE_VIS : 0u);
            check(fsr_reconstruct_files_ex(mHandle, mDirectory.c_str(), mPattern.c_str(), f, f + 1, flags, &ms,
                                           nullptr),
                  "frame " + std::to_string(f));
            mTimeConsuming.push_back(ms);
            fsr_stats st;
            fsr_get_stats(mHandle, &st);
            fsr_get_frame_header(mHandle, &mHeader);
            mNumParticles = (unsigned int)st.n_particles;
            if (mSaveCfgFile) {
                tri.push_back((double)(st.n_mesh_vertices / 3));
                spr.push_back(st.n_particles ? (double)st.n_surface_particles / st.n_particles : 0.0);
                svr.push_back(st.n_grid_vertices ? (double)st.n_band_vertices / st.n_grid_vertices : 0.0);
                // stage groups: surface extraction (hashing..band), field, marching cubes
                es.push_back(st.stage_ms[0] + st.stage_ms[1] + st.stage_ms[2] + st.stage_ms[3] + st.stage_ms[4]);
                sf.push_back(st.stage_ms[5] + st.stage_ms[6] + st.stage_ms[7]);
                mc.push_back(st.stage_ms[8] + st.stage_ms[9] + st.stage_ms[10]);
            }
        }
        saveTimeConsumingRecordToFile();
        if (mSaveCfgFile) saveConfigurationToFile(tri, spr, svr, es, sf, mc);
    }

    void setOutputMeshFile(bool flag) { mSaveObjFile = flag; }
    void setOutputConfigFile(bool flag) { mSaveCfgFile = flag; }
    void setOutputVisualizeFile(bool flag) { mSaveVisFile = flag; }
    /* Read stem.xyzb instead of parsing stem.xyz when it is current, and
     * write it after parsing (FSR_FILES_SIDECAR). */
    void setBinarySidecar(bool flag) { mSidecar = flag; }
    /* Write welded (indexed) .obj files instead of triangle soups
     * (FSR_FLAG_WELD, FSR_FILES_INDEXED_OBJ). */
    void setIndexedMesh(bool flag)
    {
        mIndexed = flag;
        mParams.flags = flag ? (mParams.flags | FSR_FLAG_WELD) : (mParams.flags & ~FSR_FLAG_WELD);
        if (mHandle) check(fsr_set_params(mHandle, &mParams), "fsr_set_params");
    }

    SimParam getSimulationParameters() const
    {
        SimParam p{};
        p.particleRadius = mHeader.particle_radius;
        p.particleMass = mHeader.particle_mass;
        p.smoothingRadius = mHeader.kernel_radius;
        p.smoothingRadiusSq = mHeader.kernel_radius * mHeader.kernel_radius;
        p.smoothingRadiusInv = mHeader.kernel_radius > 0.f ? (float)(1.0 / (double)mHeader.kernel_radius) : 0.f;
        p.lambdaForSmoothed = mParams.smoothing_lambda;
        p.anisotropicRadius = mHeader.kernel_radius * mParams.aniso_radius_over_h;
        p.isoValue = mParams.iso_value;
        p.scSpGridResRatio = mParams.grid_ratio;
        p.expandExtent = mParams.method == FSR_METHOD_YU13 ? 3u : 4u;
        p.minNumNeighbors = mParams.min_neighbors;
        p.spatialCellSizeScale = mParams.cell_size_scale;
        return p;
    }
    unsigned int getNumberOfParticles() const { return mNumParticles; }
    std::vector<double> getTimeConsumingSequence() const { return mTimeConsuming; }

    /* Not in the reference: the parameters used for every frame (defaults of
     * the reconstructor's method; change them before reconstruct()). */
    fsr_params& parameters() { return mParams; }

protected:
    void check(fsr_status s, const std::string& what)
    {
        if (s != FSR_OK) {
            const char* msg = mHandle ? fsr_last_error(mHandle) : "";
            throw Error(s, what + ": " + msg);
        }
    }

    void saveTimeConsumingRecordToFile()
    {
        if (mTimeConsuming.empty()) return;
        std::ofstream file((mDirectory + getAlgorithmType() + ".time").c_str(), std::ios::out | std::ios::app);
        if (!file) return;
        for (double t : mTimeConsuming) file << t << ' ';
        file << std::endl;
    }

    static double mean(const std::vector<double>& v)
    {
        double s = 0.0;
        for (double x : v) s += x;
        return v.empty() ? 0.0 : s / (double)v.size();
    }

    void saveConfigurationToFile(const std::vector<double>& tri, const std::vector<double>& spr,
                                 const std::vector<double>& svr, const std::vector<double>& es,
                                 const std::vector<double>& sf, const std::vector<double>& mc)
    {
        std::ofstream file((mDirectory + getAlgorithmType() + ".config").c_str());
        if (!file) return;
        const double e = mean(es), f = mean(sf), t = mean(mc);
        file << (long long)mean(tri) << std::endl;
        file << mean(spr) << std::endl;
        file << mean(svr) << std::endl;
        file << e << std::endl;
        file << e + f << std::endl;
        file << t << std::endl;
        file << e + f + t << std::endl;
    }

    std::string mDirectory, mPattern;
    unsigned int mFrom, mTo;
    int mDevice;
    bool mSaveObjFile = true, mSaveVisFile = false, mSaveCfgFile = false, mSidecar = false, mIndexed = false;
    fsr_params mParams{};
    fsr_handle* mHandle = nullptr;
    fsr_frame_header mHeader{};
    unsigned int mNumParticles = 0;
    std::vector<double> mTimeConsuming;
};

/* ReconstructorGPUOursZB05.cpp:12-15 */
class ReconstructorGPUOursZB05 final : public ReconstructorGPU {
public:
    ReconstructorGPUOursZB05(const std::string& directory, const std::string& filePattern, unsigned int from,
                             unsigned int to, int device = 0)
        : ReconstructorGPU(directory, filePattern, from, to, FSR_METHOD_ZB05, device) {}
    std::string getAlgorithmType() override { return "Our Algorithm using ZB05 kernel"; }
};

/* ReconstructorGPUOursYu13.cpp:8 */
class ReconstructorGPUOursYu13 final : public ReconstructorGPU {
public:
    ReconstructorGPUOursYu13(const std::string& directory, const std::string& filePattern, unsigned int from,
                             unsigned int to, int device = 0)
        : ReconstructorGPU(directory, filePattern, from, to, FSR_METHOD_YU13, device) {}
    std::string getAlgorithmType() override { return "Our Algorithm using anisotropic kernel"; }
};

/* ReconstructorGPUAkinci12.cpp:20-23 */
class ReconstructorGPUAkinci12 final : public ReconstructorGPU {
public:
    ReconstructorGPUAkinci12(const std::string& directory, const std::string& filePattern, unsigned int from,
                             unsigned int to, int device = 0)
        : ReconstructorGPU(directory, filePattern, from, to, FSR_METHOD_AKINCI12, device) {}
    std::string getAlgorithmType() override { return "Akinci12 using ZB05 kernel"; }
};

/* The TC01 field (ReconstructionCUDA.cu:178-227) has no reconstructor class
 * in the reference; this one runs it on the ZB05 pipeline. */
class ReconstructorGPUOursTC01 final : public ReconstructorGPU {
public:
    ReconstructorGPUOursTC01(const std::string& directory, const std::string& filePattern, unsigned int from,
                             unsigned int to, int device = 0)
        : ReconstructorGPU(directory, filePattern, from, to, FSR_METHOD_TC01, device) {}
    std::string getAlgorithmType() override { return "Our Algorithm using TC01 kernel"; }
};

}  // namespace fsr_gb300

#endif
