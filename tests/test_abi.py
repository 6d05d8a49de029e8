"""The C-ABI library loads on a machine without a GPU and exports every
entry point the public headers declare; host-only calls work."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib():
    from fluidsurfacereconstructiongpu_gb300 import build
    if not os.path.exists(build.LIB_PATH):
        build.build()
    from fluidsurfacereconstructiongpu_gb300 import _native
    return _native


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    names = set(re.findall(r"\b((?:fsr_|launch|bind)[A-Za-z0-9_]*)\s*\(", src))
    return sorted(n for n in names if not n.startswith("FSR_"))


@pytest.mark.parametrize("header", sorted(h for h in os.listdir(os.path.join(ROOT, "include")) if h.endswith(".h")))
def test_every_declared_symbol_is_exported(header):
    N = _lib()
    names = _declared(header)
    assert names, header
    missing = [n for n in names if not hasattr(N.lib, n)]
    assert not missing, f"{header}: not exported: {missing}"


def test_host_only_calls():
    N = _lib()
    assert N.lib.fsr_abi_version() == 1
    assert b"sm_103a" in N.lib.fsr_build_info()
    for m in range(4):
        p = N.Params()
        assert N.lib.fsr_default_params(m, ctypes.byref(p)) == 0
    p = N.Params()
    N.lib.fsr_default_params(N.METHOD_YU13, ctypes.byref(p))
    assert abs(p.cell_size_scale - 1.3) < 1e-6 and p.grid_ratio == 3 and p.min_neighbors == 25
    assert N.lib.fsr_default_params(9, ctypes.byref(p)) == 1


def test_xyz_obj_roundtrip(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, synthetic
    fr = synthetic.format_example()
    path = str(tmp_path / "frame_000000.xyz")
    api.write_xyz(path, fr)
    hdr, xyz, den = api.read_xyz(path)
    assert np.array_equal(xyz, fr.pos) and np.array_equal(den, fr.density)
    assert hdr.kernel_radius == np.float32(0.036) and list(hdr.bbox_max) == pytest.approx([3.04, 2.04, 1.54])
    # the documented example file parses to the same numbers
    mesh = api.Mesh(positions=np.arange(18, dtype=np.float32).reshape(6, 3) / 7,
                    normals=np.ones((6, 3), np.float32))
    obj = str(tmp_path / "m.obj")
    api.write_obj(obj, mesh)
    lines = open(obj).read().splitlines()
    assert lines[0].startswith("v ") and lines[6].startswith("vn ") and lines[12] == "f 1//1 2//2 3//3 "
    assert len(lines) == 6 + 6 + 2


def test_malformed_xyz_is_an_error(tmp_path):
    from fluidsurfacereconstructiongpu_gb300 import api, _native
    p = tmp_path / "bad.xyz"
    p.write_text("0 0 0\n1 1 1\n0.1\n0.01\n0.001\n0.5 0.5 oops 1000\n")
    with pytest.raises(_native.FsrError) as e:
        api.read_xyz(str(p))
    assert e.value.status == 6
    with pytest.raises(_native.FsrError) as e:
        api.read_xyz(str(tmp_path / "missing.xyz"))
    assert e.value.status == 5


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    N = _lib()
    p = N.Params()
    N.lib.fsr_default_params(0, ctypes.byref(p))
    h = ctypes.c_void_p()
    assert N.lib.fsr_create(ctypes.byref(p), 0, ctypes.byref(h)) == 3
