// File formats and the file-driven frame loop.
//   .xyz reader: data_format.txt:1-28, ReconstructorGPU::readParticlesFromFile
//                (ReconstructorGPU.cpp:200-290)
//   .obj writer: ReconstructorGPUOurs::saveFluidSurfaceObjToFile
//                (ReconstructorGPUOurs.cpp:20-100)
//   frame loop:  ReconstructorGPU::reconstruct (ReconstructorGPU.cpp:25-79)
#include <cuda_runtime.h>

#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fsr.h"
#include "fsr_internal.h"

namespace {

// Reads up to `want` floats from a line; returns how many were parsed and
// whether anything but whitespace follows.
int parse_floats(const char* s, float* out, int want, bool* trailing)
{
    int got = 0;
    const char* p = s;
    while (got < want) {
        char* end = nullptr;
        errno = 0;
        const float v = std::strtof(p, &end);
        if (end == p) break;
        out[got++] = v;
        p = end;
    }
    while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') ++p;
    if (trailing) *trailing = *p != '\0';
    return got;
}

bool blank(const char* s)
{
    for (; *s; ++s)
        if (*s != ' ' && *s != '\t' && *s != '\r' && *s != '\n') return false;
    return true;
}

struct LineReader {
    FILE* f;
    std::vector<char> buf;
    explicit LineReader(FILE* fp) : f(fp), buf(1 << 16) {}
    // false at end of file; long lines are read whole
    bool next(std::string& line)
    {
        line.clear();
        while (std::fgets(buf.data(), (int)buf.size(), f)) {
            line += buf.data();
            if (!line.empty() && line.back() == '\n') return true;
        }
        return !line.empty();
    }
};

}  // namespace

extern "C" {

fsr_status fsr_read_xyz(const char* path, fsr_frame_header* hdr, float** xyz, float** density, uint64_t* n)
{
    if (!path || !hdr || !xyz || !density || !n) return FSR_ERR_INVALID_ARGUMENT;
    *xyz = nullptr;
    *density = nullptr;
    *n = 0;
    FILE* f = std::fopen(path, "rb");
    if (!f) return FSR_ERR_IO;
    LineReader rd(f);
    std::string line;
    float v[4];
    bool trail = false;
    fsr_frame_header h{};
    // bounding box min, max; kernel radius; particle radius; particle mass
    if (!rd.next(line) || parse_floats(line.c_str(), v, 3, &trail) != 3) { std::fclose(f); return FSR_ERR_FORMAT; }
    std::memcpy(h.bbox_min, v, sizeof(float) * 3);
    if (!rd.next(line) || parse_floats(line.c_str(), v, 3, &trail) != 3) { std::fclose(f); return FSR_ERR_FORMAT; }
    std::memcpy(h.bbox_max, v, sizeof(float) * 3);
    float* scal[3] = {&h.kernel_radius, &h.particle_radius, &h.particle_mass};
    for (int i = 0; i < 3; ++i) {
        if (!rd.next(line) || parse_floats(line.c_str(), v, 1, &trail) != 1) { std::fclose(f); return FSR_ERR_FORMAT; }
        *scal[i] = v[0];
    }
    std::vector<float> p, d;
    while (rd.next(line)) {
        if (blank(line.c_str())) continue;
        if (parse_floats(line.c_str(), v, 4, &trail) != 4 || trail) { std::fclose(f); return FSR_ERR_FORMAT; }
        p.push_back(v[0]);
        p.push_back(v[1]);
        p.push_back(v[2]);
        d.push_back(v[3]);
    }
    std::fclose(f);
    const uint64_t cnt = d.size();
    float* px = (float*)std::malloc(sizeof(float) * 3 * (cnt ? cnt : 1));
    float* pd = (float*)std::malloc(sizeof(float) * (cnt ? cnt : 1));
    if (!px || !pd) {
        std::free(px);
        std::free(pd);
        return FSR_ERR_OUT_OF_MEMORY;
    }
    if (cnt) {
        std::memcpy(px, p.data(), sizeof(float) * 3 * cnt);
        std::memcpy(pd, d.data(), sizeof(float) * cnt);
    }
    *hdr = h;
    *xyz = px;
    *density = pd;
    *n = cnt;
    return FSR_OK;
}

void fsr_free_host(void* p) { std::free(p); }

fsr_status fsr_write_obj(const char* path, const float* pos, const float* nrm, uint64_t nv)
{
    if (!path || (nv && (!pos || !nrm)) || nv % 3 != 0) return FSR_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return FSR_ERR_IO;
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    // std::ostream's default float formatting is %g with 6 significant digits
    for (uint64_t i = 0; i < nv; ++i) std::fprintf(f, "v %g %g %g\n", pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    for (uint64_t i = 0; i < nv; ++i) std::fprintf(f, "vn %g %g %g\n", nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    for (uint64_t i = 1; i <= nv; i += 3)
        std::fprintf(f, "f %llu//%llu %llu//%llu %llu//%llu \n", (unsigned long long)i, (unsigned long long)i,
                     (unsigned long long)(i + 1), (unsigned long long)(i + 1), (unsigned long long)(i + 2),
                     (unsigned long long)(i + 2));
    const bool ok = std::fflush(f) == 0;
    std::fclose(f);
    return ok ? FSR_OK : FSR_ERR_IO;
}

fsr_status fsr_reconstruct_files(fsr_handle* h, const char* directory, const char* pattern, uint32_t from,
                                 uint32_t to, int write_obj, double* frame_ms)
{
    if (!h || !directory || !pattern) return FSR_ERR_INVALID_ARGUMENT;
    if (from >= to) return FSR_ERR_INVALID_ARGUMENT;  // "Wrong settings occur for frame range."
    std::vector<float> mp, mn;
    for (uint32_t fr = from; fr < to; ++fr) {
        char base[512];
        std::snprintf(base, sizeof(base), pattern, fr);
        const std::string stem = std::string(directory) + base;
        fsr_frame_header hdr;
        float* xyz = nullptr;
        float* den = nullptr;
        uint64_t n = 0;
        fsr_status s = fsr_read_xyz((stem + ".xyz").c_str(), &hdr, &xyz, &den, &n);
        if (s != FSR_OK) {
            h->last_error = "cannot read " + stem + ".xyz";
            return s;
        }
        // upload outside the timer, as beginFrame does (ReconstructorGPU.cpp:110-118)
        const uint64_t nn = n ? n : 1;
        cudaError_t e = h->in_xyz.ensure(12ull * nn);
        if (e == cudaSuccess) e = h->in_den.ensure(4ull * nn);
        if (e == cudaSuccess && n) e = cudaMemcpy(h->in_xyz.ptr, xyz, 12ull * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && n) e = cudaMemcpy(h->in_den.ptr, den, 4ull * n, cudaMemcpyHostToDevice);
        fsr_free_host(xyz);
        fsr_free_host(den);
        if (e != cudaSuccess) {
            h->last_error = std::string("upload: ") + cudaGetErrorString(e);
            return FSR_ERR_CUDA;
        }
        // the reference's timed scope (ReconstructorGPU.cpp:46-54): hashing to mesh
        const auto t0 = std::chrono::steady_clock::now();
        s = fsr_reconstruct(h, &hdr, (const float*)h->in_xyz.ptr, (const float*)h->in_den.ptr, n, nullptr);
        const auto t1 = std::chrono::steady_clock::now();
        if (s != FSR_OK) return s;
        uint64_t nv = h->stats.n_mesh_vertices;
        if (frame_ms) frame_ms[fr - from] = std::chrono::duration<double, std::milli>(t1 - t0).count();
        if (write_obj) {
            mp.resize(3 * nv);
            mn.resize(3 * nv);
            s = fsr_copy_mesh(h, mp.data(), mn.data(), nv, &nv);
            if (s != FSR_OK) return s;
            s = fsr_write_obj((stem + ".obj").c_str(), mp.data(), mn.data(), nv);
            if (s != FSR_OK) return s;
        }
    }
    return FSR_OK;
}

}  // extern "C"
