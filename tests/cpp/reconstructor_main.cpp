// Drives the header-only reconstructor classes the way the reference's
// main program drives ReconstructorGPU: frames [from, to) of a directory,
// .obj and .config output on.  Usage: reconstructor_main <method> <dir> <pattern> <from> <to>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "fsr_reconstructor.hpp"

int main(int argc, char** argv)
{
    if (argc != 6) return 2;
    const std::string m = argv[1];
    const unsigned from = (unsigned)std::atoi(argv[4]), to = (unsigned)std::atoi(argv[5]);
    fsr_gb300::ReconstructorGPU::ptr r;
    if (m == "zb05") r.reset(new fsr_gb300::ReconstructorGPUOursZB05(argv[2], argv[3], from, to));
    else if (m == "yu13") r.reset(new fsr_gb300::ReconstructorGPUOursYu13(argv[2], argv[3], from, to));
    else if (m == "akinci12") r.reset(new fsr_gb300::ReconstructorGPUAkinci12(argv[2], argv[3], from, to));
    else if (m == "tc01") r.reset(new fsr_gb300::ReconstructorGPUOursTC01(argv[2], argv[3], from, to));
    else return 2;
    r->setOutputMeshFile(true);
    r->setOutputConfigFile(true);
    try {
        r->reconstruct();
    } catch (const fsr_gb300::Error& e) {
        std::printf("error %d %s\n", (int)e.status, e.what());
        return 1;
    }
    const SimParam p = r->getSimulationParameters();
    std::printf("type=%s\n", r->getAlgorithmType().c_str());
    std::printf("particles=%u h=%.9g ratio=%u iso=%.9g\n", r->getNumberOfParticles(), p.smoothingRadius,
                p.scSpGridResRatio, p.isoValue);
    for (double t : r->getTimeConsumingSequence()) std::printf("ms=%.6f\n", t);
    return 0;
}
