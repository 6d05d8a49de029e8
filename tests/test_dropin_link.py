"""Drop-in proof for the kernel-level ABI: the reference's own host classes
(FluidSurfaceReconstruction/GPU/ReconstructorGPU*.cpp and main.cpp),
compiled unmodified, link against libfsr_gb300.so with no undefined symbol.
Only runs where the reference sources are present; nothing is executed."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference checkout, as the oracle's build recipe resolves it (REF_ROOT)
REF = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), "--print-root"], capture_output=True,
                     text=True, check=True).stdout.strip()
SRC = os.path.join(REF, "FluidSurfaceReconstruction")
FILES = ["main.cpp"] + ["GPU/" + f for f in ("ReconstructorGPU.cpp", "ReconstructorGPUOurs.cpp",
                                             "ReconstructorGPUOursZB05.cpp", "ReconstructorGPUOursYu13.cpp",
                                             "ReconstructorGPUAkinci12.cpp", "MarchingCubesCPU.cpp",
                                             "MarchingCubesHelper.cpp", "MathVector.cpp", "Timer.cpp")]


@pytest.mark.skipif(not os.path.isdir(SRC), reason="reference sources not present")
def test_reference_host_classes_link_against_library(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import build
    lib = build.build()
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    objs = []
    for f in FILES:
        o = str(tmp_path / (os.path.basename(f) + ".o"))
        # the samples' helper_cuda.h is replaced by the oracle's two-macro shim
        subprocess.run(["g++", "-std=c++14", "-O0", "-w", "-c", "-include", "memory", "-include", "fstream",
                        "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", SRC, "-I", os.path.join(SRC, "GPU"),
                        "-I", os.path.join(REF, "include"), "-I", os.path.join(cuda, "include"),
                        os.path.join(SRC, f), "-o", o], check=True)
        objs.append(o)
    exe = str(tmp_path / "dropin")
    r = subprocess.run(["g++", "-o", exe] + objs + [lib, "-L" + os.path.join(cuda, "lib64"), "-lcudart",
                                                      "-Wl,--no-undefined"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(exe)
