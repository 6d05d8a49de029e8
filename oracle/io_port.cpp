// CPU baseline for the file formats.  TEST INFRASTRUCTURE ONLY: the I/O leg of
// the benchmark times it beside the library's reader and writer; the product
// never links or calls it.
//
// A restatement of the reference's stream-based file code, one thread:
//  - reader: ReconstructorGPU::readParticlesFromFile (ReconstructorGPU.cpp:
//    200-290): std::getline per line, a std::stringstream per line and
//    operator>> for each float, particles appended to vectors;
//  - writer: ReconstructorGPUOurs::saveFluidSurfaceObjToFile
//    (ReconstructorGPUOurs.cpp:58-99): std::ofstream, operator<< for every
//    number and std::endl (a flush) after every line.
// Blank or malformed lines are skipped here (the reference appends whatever
// the stream left in the variables).
#include <cstdint>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

extern "C" {

// Reads an .xyz file into out (n x 4 floats: x, y, z, density) and hdr (9
// floats); returns the particle count, or -1 if the file cannot be opened,
// or -(count + 2) when out holds fewer than count particles.
int64_t io_port_read_xyz(const char* path, float* hdr, float* out, int64_t capacity)
{
    std::ifstream file(path);
    if (!file) return -1;
    std::string line;
    int k = 0;
    for (int l = 0; l < 5; ++l) {
        std::getline(file, line);
        std::stringstream ss;
        ss << line;
        const int cnt = l < 2 ? 3 : 1;
        for (int c = 0; c < cnt; ++c) ss >> hdr[k++];
    }
    std::vector<float> v;
    while (std::getline(file, line)) {
        std::stringstream str;
        str << line;
        float a, b, c, d;
        if (str >> a >> b >> c >> d) {
            v.push_back(a);
            v.push_back(b);
            v.push_back(c);
            v.push_back(d);
        }
    }
    const int64_t n = (int64_t)(v.size() / 4);
    if (n > capacity) return -(n + 2);
    for (size_t i = 0; i < v.size(); ++i) out[i] = v[i];
    return n;
}

// Writes the triangle soup as .obj; returns 0, or -1 if the file cannot be
// opened.
int io_port_write_obj(const char* path, const float* pos, const float* nrm, int64_t nv)
{
    std::ofstream file(path);
    if (!file) return -1;
    for (int64_t i = 0; i < nv; ++i)
        file << "v " << pos[3 * i] << " " << pos[3 * i + 1] << " " << pos[3 * i + 2] << std::endl;
    for (int64_t i = 0; i < nv; ++i)
        file << "vn " << nrm[3 * i] << " " << nrm[3 * i + 1] << " " << nrm[3 * i + 2] << std::endl;
    for (int64_t i = 1; i <= nv; i += 3) {
        file << "f ";
        file << (i + 0) << "//" << (i + 0) << " ";
        file << (i + 1) << "//" << (i + 1) << " ";
        file << (i + 2) << "//" << (i + 2) << " ";
        file << std::endl;
    }
    return 0;
}

}  // extern "C"
