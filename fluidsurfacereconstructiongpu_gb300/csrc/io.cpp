// File formats and the file-driven frame loop.
//   .xyz reader: data_format.txt:1-28, ReconstructorGPU::readParticlesFromFile
//                (ReconstructorGPU.cpp:200-290)
//   .obj writer: ReconstructorGPUOurs::saveFluidSurfaceObjToFile
//                (ReconstructorGPUOurs.cpp:20-100)
//   frame loop:  ReconstructorGPU::reconstruct (ReconstructorGPU.cpp:25-79)
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <charconv>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fsr.h"
#include "fsr_internal.h"

namespace {

std::atomic<uint32_t> g_io_threads{0};

uint32_t io_threads()
{
    const uint32_t t = g_io_threads.load();
    if (t) return t;
    const uint32_t hw = std::thread::hardware_concurrency();
    return std::max(1u, std::min(hw ? hw : 1u, 64u));
}

// Runs f(k) for k in [0, parts) on up to io_threads() threads.
template <class F>
void parallel_for(uint32_t parts, F&& f)
{
    const uint32_t nt = std::min(parts, io_threads());
    if (nt <= 1) {
        for (uint32_t k = 0; k < parts; ++k) f(k);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    auto worker = [&]() {
        for (uint32_t k = next++; k < parts; k = next++) f(k);
    };
    for (uint32_t t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

// One number at p (no leading white space), as strtof parses it: the
// longest prefix that forms a float.  Decimal input goes through
// std::from_chars (correctly rounded, like strtof); anything it might read
// differently (a leading '+', hex, out-of-range values, a letter right after
// the digits) is handed to strtof on a NUL-terminated copy of the token.
bool parse_number(const char* p, const char* e, float* v, const char** next)
{
    const char* q = p;
    const bool plus = *q == '+';
    if (plus) ++q;
    if (q < e && !(plus && (*q == '-' || *q == '+'))) {
        const auto r = std::from_chars(q, e, *v, std::chars_format::general);
        if (r.ec == std::errc() && r.ptr > q) {
            const char c = r.ptr < e ? *r.ptr : ' ';
            const bool alnum = (c >= '0' && c <= '9') || (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || c == '.';
            if (!alnum) {
                *next = r.ptr;
                return true;
            }
        }
    }
    char tmp[128];
    size_t len = 0;
    while (p + len < e && !is_space(p[len]) && len + 1 < sizeof(tmp)) {
        tmp[len] = p[len];
        ++len;
    }
    tmp[len] = '\0';
    char* end = nullptr;
    errno = 0;
    *v = std::strtof(tmp, &end);
    if (end == tmp) return false;
    *next = p + (end - tmp);
    return true;
}

// Reads up to `want` numbers from the line [p, e); returns how many were
// parsed and whether anything but white space follows them.
int parse_floats(const char* p, const char* e, float* out, int want, bool* trailing)
{
    int got = 0;
    while (got < want) {
        while (p < e && is_space(*p)) ++p;
        if (p == e) break;
        const char* nx = nullptr;
        if (!parse_number(p, e, out + got, &nx)) break;
        ++got;
        p = nx;
    }
    while (p < e && is_space(*p)) ++p;
    if (trailing) *trailing = p != e;
    return got;
}

bool blank(const char* p, const char* e)
{
    for (; p < e; ++p)
        if (!is_space(*p)) return false;
    return true;
}

bool read_file(const char* path, std::vector<char>& buf)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    bool ok = std::fseek(f, 0, SEEK_END) == 0;
    const long sz = ok ? std::ftell(f) : -1;
    ok = ok && sz >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
    if (ok) {
        buf.resize((size_t)sz + 1);
        ok = std::fread(buf.data(), 1, (size_t)sz, f) == (size_t)sz;
        buf[(size_t)sz] = '\0';
        buf.resize((size_t)sz);
    }
    std::fclose(f);
    return ok;
}

// Size and modification time (ns) of a file; false if it does not exist.
bool file_stamp(const char* path, uint64_t* size, int64_t* mtime_ns)
{
    struct stat st;
    if (stat(path, &st) != 0) return false;
    *size = (uint64_t)st.st_size;
    *mtime_ns = (int64_t)st.st_mtim.tv_sec * 1000000000ll + (int64_t)st.st_mtim.tv_nsec;
    return true;
}

// .xyzb: the binary sidecar of an .xyz file.
struct XyzbHeader {
    char magic[8];        // "FSRXYZB1"
    uint64_t n;           // particles
    uint64_t src_size;    // size of the .xyz it was made from (0: none)
    int64_t src_mtime_ns; // and its modification time
    float hdr[9];         // bbox min, bbox max, h, particle radius, particle mass
    uint32_t pad[3];
};
static_assert(sizeof(XyzbHeader) == 80, "xyzb header layout");
constexpr char kXyzbMagic[8] = {'F', 'S', 'R', 'X', 'Y', 'Z', 'B', '1'};

fsr_status write_xyzb(const char* path, const fsr_frame_header* hdr, const float* xyz, const float* den, uint64_t n,
                      uint64_t src_size, int64_t src_mtime_ns)
{
    XyzbHeader h{};
    std::memcpy(h.magic, kXyzbMagic, 8);
    h.n = n;
    h.src_size = src_size;
    h.src_mtime_ns = src_mtime_ns;
    std::memcpy(h.hdr, hdr->bbox_min, 12);
    std::memcpy(h.hdr + 3, hdr->bbox_max, 12);
    h.hdr[6] = hdr->kernel_radius;
    h.hdr[7] = hdr->particle_radius;
    h.hdr[8] = hdr->particle_mass;
    // write to a temporary name and rename, so a reader never sees half a file
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return FSR_ERR_IO;
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
    if (n) {
        ok = ok && std::fwrite(xyz, 12, n, f) == n;
        ok = ok && std::fwrite(den, 4, n, f) == n;
    }
    ok = std::fclose(f) == 0 && ok;
    if (ok) ok = std::rename(tmp.c_str(), path) == 0;
    if (!ok) std::remove(tmp.c_str());
    return ok ? FSR_OK : FSR_ERR_IO;
}

fsr_status read_xyzb(const char* path, fsr_frame_header* hdr, float** xyz, float** density, uint64_t* n,
                     XyzbHeader* out_h)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return FSR_ERR_IO;
    XyzbHeader h;
    if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kXyzbMagic, 8) != 0 ||
        h.n > (1ull << 40)) {
        std::fclose(f);
        return FSR_ERR_FORMAT;
    }
    const uint64_t nn = h.n ? h.n : 1;
    float* px = (float*)std::malloc(12 * nn);
    float* pd = (float*)std::malloc(4 * nn);
    if (!px || !pd) {
        std::free(px);
        std::free(pd);
        std::fclose(f);
        return FSR_ERR_OUT_OF_MEMORY;
    }
    bool ok = true;
    if (h.n) {
        ok = std::fread(px, 12, h.n, f) == h.n;
        ok = ok && std::fread(pd, 4, h.n, f) == h.n;
    }
    std::fclose(f);
    if (!ok) {
        std::free(px);
        std::free(pd);
        return FSR_ERR_FORMAT;
    }
    std::memcpy(hdr->bbox_min, h.hdr, 12);
    std::memcpy(hdr->bbox_max, h.hdr + 3, 12);
    hdr->kernel_radius = h.hdr[6];
    hdr->particle_radius = h.hdr[7];
    hdr->particle_mass = h.hdr[8];
    *xyz = px;
    *density = pd;
    *n = h.n;
    if (out_h) *out_h = h;
    return FSR_OK;
}

// Appends printf("%g") of x: std::to_chars with the general format and
// precision 6 is specified as printf's conversion in the "C" locale, which
// is what std::ostream's default float output gives.
inline char* put_g(char* o, float x)
{
    return std::to_chars(o, o + 32, x, std::chars_format::general, 6).ptr;
}

inline char* put_u(char* o, uint64_t v) { return std::to_chars(o, o + 24, v).ptr; }

}  // namespace

extern "C" {

void fsr_io_set_threads(uint32_t n) { g_io_threads.store(std::min(n, 256u)); }

fsr_status fsr_read_xyz(const char* path, fsr_frame_header* hdr, float** xyz, float** density, uint64_t* n)
{
    if (!path || !hdr || !xyz || !density || !n) return FSR_ERR_INVALID_ARGUMENT;
    *xyz = nullptr;
    *density = nullptr;
    *n = 0;
    std::vector<char> buf;
    if (!read_file(path, buf)) return FSR_ERR_IO;
    const char* p = buf.data();
    const char* const e = p + buf.size();
    auto next_line = [&](const char*& b, const char*& le) -> bool {
        if (p >= e) return false;
        b = p;
        le = (const char*)std::memchr(p, '\n', (size_t)(e - p));
        if (!le) le = e;
        p = le < e ? le + 1 : e;
        return true;
    };
    float v[4];
    bool trail = false;
    fsr_frame_header h{};
    const char *lb, *le;
    // bounding box min, max; kernel radius; particle radius; particle mass
    if (!next_line(lb, le) || parse_floats(lb, le, v, 3, &trail) != 3) return FSR_ERR_FORMAT;
    std::memcpy(h.bbox_min, v, sizeof(float) * 3);
    if (!next_line(lb, le) || parse_floats(lb, le, v, 3, &trail) != 3) return FSR_ERR_FORMAT;
    std::memcpy(h.bbox_max, v, sizeof(float) * 3);
    float* scal[3] = {&h.kernel_radius, &h.particle_radius, &h.particle_mass};
    for (int i = 0; i < 3; ++i) {
        if (!next_line(lb, le) || parse_floats(lb, le, v, 1, &trail) != 1) return FSR_ERR_FORMAT;
        *scal[i] = v[0];
    }
    // the particle lines: split into chunks at line starts, count each
    // chunk's non-blank lines, then parse every chunk into its slots
    const char* body = p;
    const size_t bytes = (size_t)(e - body);
    const uint32_t parts = (uint32_t)std::max<size_t>(1, std::min<size_t>(4ull * io_threads(), bytes >> 16));
    std::vector<const char*> cut(parts + 1);
    cut[0] = body;
    cut[parts] = e;
    for (uint32_t k = 1; k < parts; ++k) {
        const char* c = body + bytes * k / parts;
        c = std::max(c, cut[k - 1]);
        const char* nl = (const char*)std::memchr(c, '\n', (size_t)(e - c));
        cut[k] = nl ? nl + 1 : e;
    }
    std::vector<uint64_t> lines(parts + 1, 0);
    parallel_for(parts, [&](uint32_t k) {
        uint64_t c = 0;
        for (const char* q = cut[k]; q < cut[k + 1];) {
            const char* nl = (const char*)std::memchr(q, '\n', (size_t)(cut[k + 1] - q));
            const char* l_end = nl ? nl : cut[k + 1];
            if (!blank(q, l_end)) ++c;
            q = nl ? nl + 1 : cut[k + 1];
        }
        lines[k + 1] = c;
    });
    for (uint32_t k = 0; k < parts; ++k) lines[k + 1] += lines[k];
    const uint64_t cnt = lines[parts];
    float* px = (float*)std::malloc(sizeof(float) * 3 * (cnt ? cnt : 1));
    float* pd = (float*)std::malloc(sizeof(float) * (cnt ? cnt : 1));
    if (!px || !pd) {
        std::free(px);
        std::free(pd);
        return FSR_ERR_OUT_OF_MEMORY;
    }
    std::atomic<bool> bad{false};
    parallel_for(parts, [&](uint32_t k) {
        uint64_t i = lines[k];
        float w[4];
        bool tr = false;
        for (const char* q = cut[k]; q < cut[k + 1] && !bad.load(std::memory_order_relaxed);) {
            const char* nl = (const char*)std::memchr(q, '\n', (size_t)(cut[k + 1] - q));
            const char* l_end = nl ? nl : cut[k + 1];
            if (!blank(q, l_end)) {
                if (parse_floats(q, l_end, w, 4, &tr) != 4 || tr) {
                    bad = true;
                    return;
                }
                px[3 * i] = w[0];
                px[3 * i + 1] = w[1];
                px[3 * i + 2] = w[2];
                pd[i] = w[3];
                ++i;
            }
            q = nl ? nl + 1 : cut[k + 1];
        }
    });
    if (bad) {
        std::free(px);
        std::free(pd);
        return FSR_ERR_FORMAT;
    }
    *hdr = h;
    *xyz = px;
    *density = pd;
    *n = cnt;
    return FSR_OK;
}

void fsr_free_host(void* p) { std::free(p); }

fsr_status fsr_write_xyz_binary(const char* path, const fsr_frame_header* hdr, const float* xyz, const float* density,
                                uint64_t n)
{
    if (!path || !hdr || (n && (!xyz || !density))) return FSR_ERR_INVALID_ARGUMENT;
    return write_xyzb(path, hdr, xyz, density, n, 0, 0);
}

fsr_status fsr_read_xyz_binary(const char* path, fsr_frame_header* hdr, float** xyz, float** density, uint64_t* n)
{
    if (!path || !hdr || !xyz || !density || !n) return FSR_ERR_INVALID_ARGUMENT;
    *xyz = nullptr;
    *density = nullptr;
    *n = 0;
    return read_xyzb(path, hdr, xyz, density, n, nullptr);
}

}  // extern "C"

namespace {

// v lines, vn lines, then f lines (face(w, t) writes triangle t's line),
// formatted in blocks of lines by all threads into per-part buffers and
// written in order.
template <class Face>
fsr_status write_obj_lines(const char* path, const float* pos, const float* nrm, uint64_t nv, uint64_t ntri,
                           Face&& face)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) return FSR_ERR_IO;
    constexpr uint64_t kLines = 1 << 15;  // lines per part
    const uint32_t nt = io_threads();
    std::vector<std::vector<char>> out(nt);
    bool ok = true;
    auto emit = [&](uint64_t count, size_t max_line, auto&& line) {
        for (uint64_t b = 0; b < count && ok; b += kLines * nt) {
            const uint32_t parts = (uint32_t)std::min<uint64_t>(nt, (count - b + kLines - 1) / kLines);
            parallel_for(parts, [&](uint32_t k) {
                const uint64_t l0 = b + k * kLines, l1 = std::min(count, l0 + kLines);
                std::vector<char>& o = out[k];
                o.resize((l1 - l0) * max_line);
                char* w = o.data();
                for (uint64_t i = l0; i < l1; ++i) w = line(w, i);
                o.resize((size_t)(w - o.data()));
            });
            for (uint32_t k = 0; k < parts && ok; ++k)
                ok = std::fwrite(out[k].data(), 1, out[k].size(), f) == out[k].size();
        }
    };
    auto vec3 = [](char* w, const char* tag, size_t tl, const float* a) {
        std::memcpy(w, tag, tl);
        w += tl;
        w = put_g(w, a[0]);
        *w++ = ' ';
        w = put_g(w, a[1]);
        *w++ = ' ';
        w = put_g(w, a[2]);
        *w++ = '\n';
        return w;
    };
    // "v x y z" / "vn x y z" with %g numbers (at most 15 characters each)
    emit(nv, 64, [&](char* w, uint64_t i) { return vec3(w, "v ", 2, pos + 3 * i); });
    emit(nv, 64, [&](char* w, uint64_t i) { return vec3(w, "vn ", 3, nrm + 3 * i); });
    emit(ntri, 2 + 6 * 22 + 8, face);
    ok = std::fclose(f) == 0 && ok;
    return ok ? FSR_OK : FSR_ERR_IO;
}

// "f a//a b//b c//c " with 1-based vertex numbers
inline char* face_line(char* w, uint64_t a, uint64_t b, uint64_t c)
{
    *w++ = 'f';
    *w++ = ' ';
    const uint64_t id[3] = {a, b, c};
    for (int k = 0; k < 3; ++k) {
        w = put_u(w, id[k]);
        *w++ = '/';
        *w++ = '/';
        w = put_u(w, id[k]);
        *w++ = ' ';
    }
    *w++ = '\n';
    return w;
}

}  // namespace

extern "C" {

fsr_status fsr_write_obj(const char* path, const float* pos, const float* nrm, uint64_t nv)
{
    if (!path || (nv && (!pos || !nrm)) || nv % 3 != 0) return FSR_ERR_INVALID_ARGUMENT;
    return write_obj_lines(path, pos, nrm, nv, nv / 3,
                           [](char* w, uint64_t t) { return face_line(w, 3 * t + 1, 3 * t + 2, 3 * t + 3); });
}

fsr_status fsr_write_obj_indexed(const char* path, const float* pos, const float* nrm, uint64_t nv,
                                 const uint32_t* idx, uint64_t ni)
{
    if (!path || (nv && (!pos || !nrm)) || (ni && !idx) || ni % 3 != 0) return FSR_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < ni; ++i)
        if (idx[i] >= nv) return FSR_ERR_INVALID_ARGUMENT;
    return write_obj_lines(path, pos, nrm, nv, ni / 3, [idx](char* w, uint64_t t) {
        return face_line(w, (uint64_t)idx[3 * t] + 1, (uint64_t)idx[3 * t + 1] + 1, (uint64_t)idx[3 * t + 2] + 1);
    });
}

}  // extern "C"

namespace {

struct LoadedFrame {
    fsr_status status = FSR_OK;
    fsr_frame_header hdr{};
    float* xyz = nullptr;
    float* den = nullptr;
    uint64_t n = 0;
    double ms = 0.0;
    std::string error;
    void release()
    {
        fsr_free_host(xyz);
        fsr_free_host(den);
        xyz = den = nullptr;
    }
};

// Reads stem.xyz, or its sidecar stem.xyzb when `sidecar` is set and the
// sidecar was made from the .xyz as it is now (same size and modification
// time); a parsed .xyz then gets a fresh sidecar.
LoadedFrame load_frame(const std::string& stem, bool sidecar)
{
    LoadedFrame f;
    const auto t0 = std::chrono::steady_clock::now();
    const std::string xyz = stem + ".xyz", xyzb = stem + ".xyzb";
    uint64_t size = 0;
    int64_t mtime = 0;
    const bool have = file_stamp(xyz.c_str(), &size, &mtime);
    bool done = false;
    if (sidecar && have) {
        XyzbHeader bh;
        if (read_xyzb(xyzb.c_str(), &f.hdr, &f.xyz, &f.den, &f.n, &bh) == FSR_OK) {
            if (bh.src_size == size && bh.src_mtime_ns == mtime) done = true;
            else f.release();
        }
    }
    if (!done) {
        f.status = fsr_read_xyz(xyz.c_str(), &f.hdr, &f.xyz, &f.den, &f.n);
        if (f.status != FSR_OK) f.error = "cannot read " + xyz;
        else if (sidecar && have) write_xyzb(xyzb.c_str(), &f.hdr, f.xyz, f.den, f.n, size, mtime);  // best effort
    }
    f.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return f;
}

}  // namespace

extern "C" {

fsr_status fsr_reconstruct_files_ex(fsr_handle* h, const char* directory, const char* pattern, uint32_t from,
                                    uint32_t to, uint32_t flags, double* frame_ms, fsr_files_timing* timing)
{
    if (!h || !directory || !pattern) return FSR_ERR_INVALID_ARGUMENT;
    if (from >= to) return FSR_ERR_INVALID_ARGUMENT;  // "Wrong settings occur for frame range."
    const auto w0 = std::chrono::steady_clock::now();
    fsr_files_timing tm{};
    const bool sidecar = (flags & FSR_FILES_SIDECAR) != 0;
    auto stem_of = [&](uint32_t fr) {
        char base[512];
        std::snprintf(base, sizeof(base), pattern, fr);
        return std::string(directory) + base;
    };
    // frame k + 1 is read while frame k runs on the GPU, and frame k's .obj
    // is written while frame k + 1 runs
    std::future<LoadedFrame> next = std::async(std::launch::async, load_frame, stem_of(from), sidecar);
    std::future<fsr_status> writer;
    std::string writer_path;
    double write_ms = 0.0;
    fsr_status st = FSR_OK;
    for (uint32_t fr = from; fr < to && st == FSR_OK; ++fr) {
        const std::string stem = stem_of(fr);
        LoadedFrame cur = next.get();
        if (fr + 1 < to) next = std::async(std::launch::async, load_frame, stem_of(fr + 1), sidecar);
        tm.read_ms += cur.ms;
        if (cur.status != FSR_OK) {
            h->last_error = cur.error;
            st = cur.status;
            break;
        }
        // upload outside the timer, as beginFrame does (ReconstructorGPU.cpp:110-118)
        const auto u0 = std::chrono::steady_clock::now();
        const uint64_t n = cur.n, nn = n ? n : 1;
        cudaError_t e = h->in_xyz.ensure(12ull * nn);
        if (e == cudaSuccess) e = h->in_den.ensure(4ull * nn);
        if (e == cudaSuccess && n) e = cudaMemcpy(h->in_xyz.ptr, cur.xyz, 12ull * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && n) e = cudaMemcpy(h->in_den.ptr, cur.den, 4ull * n, cudaMemcpyHostToDevice);
        cur.release();
        tm.upload_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - u0).count();
        if (e != cudaSuccess) {
            h->last_error = std::string("upload: ") + cudaGetErrorString(e);
            st = FSR_ERR_CUDA;
            break;
        }
        // the reference's timed scope (ReconstructorGPU.cpp:46-54): hashing to mesh
        const auto t0 = std::chrono::steady_clock::now();
        st = fsr_reconstruct(h, &cur.hdr, (const float*)h->in_xyz.ptr, (const float*)h->in_den.ptr, n, nullptr);
        const auto t1 = std::chrono::steady_clock::now();
        if (st != FSR_OK) break;
        const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        tm.reconstruct_ms += ms;
        if (frame_ms) frame_ms[fr - from] = ms;
        if (flags & FSR_FILES_WRITE_VIS) {
            // after the timed scope, as ReconstructorGPU::reconstruct does (cpp:57-61)
            char base[512];
            std::snprintf(base, sizeof(base), pattern, fr);
            st = fsr_write_vis(h, (stem + ".vis").c_str(), (std::string(base) + ".obj").c_str());
            if (st != FSR_OK) {
                if (h->last_error.empty()) h->last_error = "cannot write " + stem + ".vis";
                break;
            }
        }
        if (flags & FSR_FILES_WRITE_OBJ) {
            const bool indexed = (flags & FSR_FILES_INDEXED_OBJ) != 0;
            uint64_t nv = indexed ? h->stats.n_weld_vertices : h->stats.n_mesh_vertices;
            uint64_t ni = indexed ? h->stats.n_mesh_vertices : 0;
            auto mp = std::make_shared<std::vector<float>>(3 * nv);
            auto mn = std::make_shared<std::vector<float>>(3 * nv);
            auto mi = std::make_shared<std::vector<uint32_t>>(ni);
            st = indexed ? fsr_copy_indexed_mesh(h, mp->data(), mn->data(), nv, mi->data(), ni, &nv, &ni)
                         : fsr_copy_mesh(h, mp->data(), mn->data(), nv, &nv);
            if (st != FSR_OK) break;
            if (writer.valid()) {
                st = writer.get();
                if (st != FSR_OK) {
                    h->last_error = "cannot write " + writer_path;
                    break;
                }
            }
            writer_path = stem + ".obj";
            writer = std::async(std::launch::async, [mp, mn, mi, nv, ni, indexed, path = writer_path, &write_ms]() {
                const auto a = std::chrono::steady_clock::now();
                const fsr_status s = indexed
                                         ? fsr_write_obj_indexed(path.c_str(), mp->data(), mn->data(), nv, mi->data(), ni)
                                         : fsr_write_obj(path.c_str(), mp->data(), mn->data(), nv);
                write_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
                return s;
            });
        }
    }
    if (next.valid()) {
        LoadedFrame rest = next.get();  // a read still in flight after an error
        rest.release();
    }
    if (writer.valid()) {
        const fsr_status s = writer.get();
        if (st == FSR_OK && s != FSR_OK) {
            h->last_error = "cannot write " + writer_path;
            st = s;
        }
    }
    tm.write_ms = write_ms;
    tm.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    if (timing) *timing = tm;
    return st;
}

fsr_status fsr_reconstruct_files(fsr_handle* h, const char* directory, const char* pattern, uint32_t from,
                                 uint32_t to, int write_obj, double* frame_ms)
{
    return fsr_reconstruct_files_ex(h, directory, pattern, from, to, write_obj ? FSR_FILES_WRITE_OBJ : 0u, frame_ms,
                                    nullptr);
}

}  // extern "C"
