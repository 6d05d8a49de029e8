// The .vis debug dump of a frame: the intermediates the reference's viewer
// reads, in its text layout (saveMiddleDataToVisFile:
// ReconstructorGPUOursZB05.cpp:104-230, ReconstructorGPUOursYu13.cpp:285-420,
// ReconstructorGPUAkinci12.cpp:290-420).  Numbers as std::ostream prints
// them (%g for floats).  Only the file is produced; the viewer itself is not
// part of this library.
#include <cuda_runtime.h>

#include <charconv>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/fsr.h"
#include "fsr_internal.h"

namespace {

struct Text {
    std::string s;
    void f(float x)
    {
        char b[32];
        s.append(b, std::to_chars(b, b + sizeof(b), x, std::chars_format::general, 6).ptr);
    }
    void u(uint64_t x)
    {
        char b[24];
        s.append(b, std::to_chars(b, b + sizeof(b), x).ptr);
    }
    void c(char ch) { s.push_back(ch); }
    void str(const char* t) { s.append(t); }
    void f3(const float* v)
    {
        f(v[0]);
        c(' ');
        f(v[1]);
        c(' ');
        f(v[2]);
        c('\n');
    }
    void u3(const uint32_t* v)
    {
        u(v[0]);
        c(' ');
        u(v[1]);
        c(' ');
        u(v[2]);
        c('\n');
    }
    // "count\n", then "i " per entry and a line break when the list is not empty
    void list(const std::vector<uint32_t>& v, bool break_if_empty = false)
    {
        u(v.size());
        c('\n');
        for (uint32_t x : v) {
            u(x);
            c(' ');
        }
        if (!v.empty() || break_if_empty) c('\n');
    }
};

template <class T>
cudaError_t fetch(std::vector<T>& out, const void* src, size_t count)
{
    out.resize(count);
    return count ? cudaMemcpy(out.data(), src, sizeof(T) * count, cudaMemcpyDeviceToHost) : cudaSuccess;
}

}  // namespace

extern "C" fsr_status fsr_write_vis(fsr_handle* h, const char* path, const char* mesh_name)
{
    if (!h || !path || !mesh_name) return FSR_ERR_INVALID_ARGUMENT;
    if (!h->frame_ready) return FSR_ERR_NOT_READY;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(h->device);
    const fsr_params& p = h->params;
    const bool yu13 = p.method == FSR_METHOD_YU13, akinci = p.method == FSR_METHOD_AKINCI12;
    fsr::Grid sp{}, sc{};
    float sp_max[3];
    uint64_t C = 0, V = 0;
    fsr::derive_grids(h->hdr_last, p, sp, sc, sp_max, C, V);
    const uint64_t n = h->n_last;
    const fsr_stats& st = h->stats;
    std::vector<float> sorted4, smooth4;
    std::vector<uint8_t> occ, surf, invol, psurf;
    std::vector<uint32_t> skeys, band, valid;
    cudaError_t e = fetch(sorted4, h->sorted.ptr, 4 * n);
    if (e == cudaSuccess) e = fetch(occ, h->occ.ptr, C);
    if (e == cudaSuccess) e = fetch(skeys, h->skeys_ptr, n);
    if (e == cudaSuccess) e = fetch(band, h->sv.ptr, st.n_band_vertices);
    if (e == cudaSuccess) e = fetch(valid, h->valid.ptr, st.n_valid_cubes);
    if (e == cudaSuccess && akinci) e = fetch(psurf, h->psurf.ptr, n);
    if (e == cudaSuccess && !akinci) e = fetch(surf, h->surf.ptr, C);
    if (e == cudaSuccess && yu13) e = fetch(smooth4, h->smoothed.ptr, 4 * n);
    if (e == cudaSuccess && yu13) e = fetch(invol, h->invol.ptr, C);
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        h->last_error = std::string("vis: ") + cudaGetErrorString(e);
        return FSR_ERR_CUDA;
    }
    Text t;
    t.s.reserve(64 * n + 12 * (C / 8 + st.n_band_vertices) + 4096);
    // spatial hashing grid: min, max (bounding box expanded by one cell), resolution, cell size
    t.f3(sp.min);
    t.f3(sp_max);
    t.u3(sp.res);
    t.f(sp.cs);
    t.c('\n');
    // scalar field grid: the same box (ReconstructorGPU.cpp:99-105)
    t.f3(sc.min);
    t.f3(sp_max);
    t.u3(sc.res);
    t.f(sc.cs);
    t.c('\n');
    t.f(h->hdr_last.particle_radius);
    t.c('\n');
    // particles in cell order
    t.u(n);
    t.c('\n');
    for (uint64_t i = 0; i < n; ++i) t.f3(&sorted4[4 * i]);
    // occupied cells; the line break follows even an empty list
    std::vector<uint32_t> lst;
    for (uint64_t c = 0; c < C; ++c)
        if (occ[c]) lst.push_back((uint32_t)c);
    t.list(lst, C > 0);
    // smoothed particles (Yu13), none for the other fields
    if (yu13) {
        t.u(n);
        t.c('\n');
        for (uint64_t i = 0; i < n; ++i) t.f3(&smooth4[4 * i]);
    } else {
        t.str("0\n");
    }
    // band vertices of the scalar grid
    t.list(band);
    // surface particles (cell order)
    lst.clear();
    for (uint64_t i = 0; i < n; ++i)
        if (akinci ? psurf[i] != 0 : surf[skeys[i]] != 0) lst.push_back((uint32_t)i);
    t.list(lst);
    // involved particles (Yu13: particles of involved cells), none for the others
    if (yu13) {
        lst.clear();
        for (uint64_t i = 0; i < n; ++i)
            if (invol[skeys[i]]) lst.push_back((uint32_t)i);
        t.list(lst);
    } else {
        t.str("0\n");
    }
    // valid cubes: positions in the band list
    t.list(valid);
    t.str(mesh_name);
    t.c('\n');
    t.f(h->hdr_last.kernel_radius);
    t.c('\n');
    FILE* f = std::fopen(path, "wb");
    if (!f) return FSR_ERR_IO;
    bool ok = std::fwrite(t.s.data(), 1, t.s.size(), f) == t.s.size();
    ok = std::fclose(f) == 0 && ok;
    return ok ? FSR_OK : FSR_ERR_IO;
}
