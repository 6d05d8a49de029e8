"""The reference's kernel-level ABI (include/fsr_compat.h) on the GPU.

Drives the launch* entry points in the order and with the buffers of the
reference's host classes (ReconstructorGPUOursZB05.cpp:22-78,
ReconstructorGPUOursYu13.cpp:24-63, ReconstructorGPUAkinci12.cpp:34-84;
launch shapes from calcGridDimBlockDim, CudaUtils.h:87-106), through ctypes
with the reference's struct layouts (Defines.h), and compares every stage
with the FP32 oracle on the same particles.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_reference_flow(method, fr, **kw):
    """Stage outputs of one frame through the compatibility layer's launch*
    entry points (oracle/ref_gpu/flow.py)."""
    from oracle import pipeline as P
    from oracle.ref_gpu import flow
    L = flow.launchers("compat")
    flow.bind_tables(L)
    params = P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass, **kw)
    out, _ = flow.frame(L, method, fr, params)
    return out


@pytest.mark.parametrize("method", ["zb05", "yu13", "akinci"])
def test_reference_abi_flow_matches_oracle(method):
    from fluidsurfacereconstructiongpu_gb300 import synthetic
    from oracle import pipeline as P
    fr = synthetic.lattice_cube(12, 0.0125, seed=1, origin=(0.3, 0.3, 0.3))
    got = _run_reference_flow(method, fr)
    prm = P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass)
    o = P.run_frame("oracle32", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, prm)
    o64 = P.run_frame("oracle64", fr.pos, fr.density, fr.bbox_min, fr.bbox_max, prm)
    assert np.array_equal(got["pos"], o.pos)
    assert np.array_equal(got["ranges"], o.ranges)
    assert np.array_equal(got["sflag"], o.sflag)
    assert np.array_equal(got["is_surf"], o.is_surf)
    assert np.array_equal(got["sv"], o.sv)
    if method == "yu13":
        assert np.array_equal(got["ninv"], o.ninv)
        assert np.array_equal(got["mean"], o.mean32)
        assert np.array_equal(got["inv"], o.inv)
        rel = np.linalg.norm(got["G"] - o64.G, axis=1) / np.linalg.norm(o64.G, axis=1)
        assert rel.max() <= 1e-5
    phi, ref = got["phi"][o.sv].astype(np.float64), o64.phi[o.sv]
    tol = (1e-5 * np.maximum(fr.h, np.abs(ref))) if method != "yu13" else 1e-5 * np.maximum(1.0, np.abs(ref))
    assert np.all(np.abs(phi - ref) <= tol)
    assert np.array_equal(got["valid"], o.valid)
    if method != "akinci":
        assert np.array_equal(got["nverts"], o.nverts)
        m64 = P.marching_cubes_on("oracle64", o, got["phi"][o.sv])
        assert got["mesh_pos"].shape == m64.mesh_pos.shape
        assert np.max(np.abs(got["mesh_pos"] - m64.mesh_pos)) <= 1e-5
