"""The header-only C++ reconstructor classes (include/fsr_reconstructor.hpp).

CPU: the header compiles and a driver program links against the library.
GPU: the driver reconstructs two .xyz frames and writes the .obj, .time and
.config files of the reference's file-driven loop; the meshes match the
Python API's on the same files.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tests", "_build")
EXE = os.path.join(BUILD, "reconstructor_main")


def _cuda_include():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return os.path.join(home, "include")


def _build():
    from fluidsurfacereconstructiongpu_gb300 import build as B
    os.makedirs(BUILD, exist_ok=True)
    lib_dir = os.path.dirname(B.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", _cuda_include(),
           os.path.join(ROOT, "tests", "cpp", "reconstructor_main.cpp"), "-o", EXE, "-L", lib_dir, "-lfsr_gb300",
           f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return EXE


def test_header_compiles_and_links():
    assert os.path.exists(_build())


@pytest.mark.gpu
def test_file_driven_loop(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    exe = _build()
    frames = [synthetic.lattice_cube(14, 0.0125, seed=s, origin=(0.3, 0.3, 0.3)) for s in (1, 2)]
    for k, fr in enumerate(frames):
        api.write_xyz(str(tmp_path / f"frame_{k:03d}.xyz"), fr)
    out = subprocess.run([exe, "zb05", str(tmp_path) + "/", "frame_%03d", "0", "2"], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.splitlines()
    assert lines[0] == "type=Our Algorithm using ZB05 kernel"
    assert sum(1 for l in lines if l.startswith("ms=")) == 2
    assert (tmp_path / "Our Algorithm using ZB05 kernel.time").exists()
    cfg = (tmp_path / "Our Algorithm using ZB05 kernel.config").read_text().split()
    assert len(cfg) == 7
    for k in range(2):
        obj = (tmp_path / f"frame_{k:03d}.obj").read_text().splitlines()
        nv = sum(1 for l in obj if l.startswith("v "))
        hdr, xyz, den = api.read_xyz(str(tmp_path / f"frame_{k:03d}.xyz"))
        with api.Reconstructor("zb05", 0) as rec:
            m = rec.reconstruct_host(xyz, den, hdr)
        assert nv == m.positions.shape[0]
        v = np.array([[float(t) for t in l.split()[1:4]] for l in obj if l.startswith("v ")], np.float32)
        assert np.allclose(v, m.positions, rtol=1e-5, atol=1e-6)
