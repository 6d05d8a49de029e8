"""The reference's kernel-level ABI (include/fsr_compat.h) on the GPU.

Drives the launch* entry points in the order and with the buffers of the
reference's host classes (ReconstructorGPUOursZB05.cpp:22-78,
ReconstructorGPUOursYu13.cpp:24-63, ReconstructorGPUAkinci12.cpp:34-84;
launch shapes from calcGridDimBlockDim, CudaUtils.h:87-106), through ctypes
with the reference's struct layouts (Defines.h), and compares every stage
with the FP32 oracle on the same particles.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

c_uint, c_float, c_ull, c_vp = ctypes.c_uint, ctypes.c_float, ctypes.c_ulonglong, ctypes.c_void_p


class dim3(ctypes.Structure):
    _fields_ = [("x", c_uint), ("y", c_uint), ("z", c_uint)]


class uint3(ctypes.Structure):
    _fields_ = [("x", c_uint), ("y", c_uint), ("z", c_uint)]


class float3(ctypes.Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float)]


class GridT(ctypes.Structure):  # Grid<T>, Defines.h:35-42
    _fields_ = [("grid", c_vp), ("size", c_ull), ("count", c_ull), ("resolution", uint3)]


class GridInfoC(ctypes.Structure):  # GridInfo, Defines.h:62-68
    _fields_ = [("minPos", float3), ("maxPos", float3), ("cellSize", c_float), ("resolution", uint3)]


def dims(n):
    """calcGridDimBlockDim (CudaUtils.h:87-106)."""
    blocks = (n + 127) // 128
    g = dim3(blocks, 1, 1)
    if blocks > 65535:
        g = dim3(65535, (blocks + 65534) // 65535, 1)
    return g, dim3(128, 1, 1)


def grid(t, res=None):
    """Grid<T> view of a tensor: a 3D grid when res is given, else a 1D array
    (rows of 3 floats count as one element each)."""
    if res is not None:
        n = res[0] * res[1] * res[2]
        r = uint3(*res)
    elif t.dim() >= 2 and t.shape[-1] == 3:
        n = t.shape[0]
        r = uint3(n, 1, 1)
    else:
        n = t.numel()
        r = uint3(n, 1, 1)
    return GridT(t.data_ptr(), n, n, r)


def ginfo(o):
    g = GridInfoC()
    g.minPos = float3(*o.minPos)
    g.maxPos = float3(*o.maxPos)
    g.cellSize = o.cellSize
    g.resolution = uint3(*o.res)
    return g


def _bind():
    """Compiles tests/compat_driver.cpp (pointer-taking wrappers that call the
    launchers with by-value structs from C++) and returns a proxy whose
    methods accept the structs and pass them by reference."""
    import os
    import subprocess
    from fluidsurfacereconstructiongpu_gb300 import _native as N  # noqa: F401  (builds/loads the library)
    from fluidsurfacereconstructiongpu_gb300.build import LIB_PATH
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    out_dir = os.path.join(here, "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "libcompat_driver.so")
    src = os.path.join(here, "compat_driver.cpp")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(LIB_PATH)):
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-o", so, src, "-I", os.path.join(root, "include"),
                        "-I", cuda_inc, LIB_PATH, "-Wl,-rpath," + os.path.dirname(LIB_PATH)], check=True)
    drv = ctypes.CDLL(so)
    drv.w_launchThrustExclusivePrefixSumScan.restype = c_uint
    drv.w_launchThrustExclusivePrefixSumScan.argtypes = [c_vp, c_vp, c_uint]

    class Proxy:
        def __getattr__(self, name):
            f = getattr(drv, "w_" + name)
            if name == "launchThrustExclusivePrefixSumScan":
                return f

            def call(*args):
                conv = [ctypes.byref(a) if isinstance(a, ctypes.Structure) else a for a in args]
                return f(*conv)
            return call
    return Proxy()


def _run_reference_flow(method, fr, **kw):
    """Returns a dict of stage outputs produced through the compat ABI."""
    import torch
    from oracle import pipeline as P
    L = _bind()
    params = P.FrameParams(method=method, h=fr.h, particle_radius=fr.particle_radius, mass=fr.mass, **kw)
    prm = params.simparam()
    iso, ratio, scale, _ = params.resolved()
    sp, sc = P.grid_derive(fr.bbox_min, fr.bbox_max, fr.h, scale, ratio)
    spi, sci = ginfo(sp), ginfo(sc)
    C, V, n = sp.count, sc.count, fr.n
    dev = "cuda"
    u32 = torch.int32
    parts = torch.from_numpy(fr.pos.copy()).to(dev)
    dens = torch.from_numpy(fr.density.copy()).to(dev)
    ranges = torch.zeros((C, 2), dtype=u32, device=dev)
    flag = torch.zeros(C, dtype=torch.float32, device=dev)
    L.launchSpatialGridBuilding(grid(parts), grid(dens), n, grid(ranges, sp.resolution), grid(flag, sp.resolution),
                                spi)
    out = dict(pos=parts.cpu().numpy(), ranges=ranges.cpu().numpy().view(np.uint32))
    L.bindTextures()

    sflag = torch.zeros(n, dtype=u32, device=dev)
    band = torch.zeros(V, dtype=u32, device=dev)
    gC = grid(ranges, sp.resolution)
    gd = dims(C)
    if method == "yu13":
        ninv = torch.zeros(C, dtype=u32, device=dev)
        L.launchExtractionOfSurfaceAndInvolveParticles(*gd, prm, grid(flag, sp.resolution),
                                                       grid(ninv, sp.resolution), grid(sflag), gC)
        out["ninv"] = ninv.cpu().numpy().view(np.uint32)
    elif method == "akinci":
        L.launchExtractionOfSurfaceParticlesForAkinci(*dims(n), prm, grid(parts), grid(dens), gC, spi, grid(sflag))
    else:
        L.launchExtractionOfSurfaceParticles(*gd, prm, grid(flag, sp.resolution), grid(sflag), gC)
    out["sflag"] = sflag.cpu().numpy().view(np.uint32)
    L.launchEstimationOfSurfaceVertices(*dims(n), prm, sci, grid(parts), grid(sflag), gC, grid(band, sc.resolution))
    out["is_surf"] = band.cpu().numpy().view(np.uint32)
    band_scan = torch.zeros(V, dtype=u32, device=dev)

    field = torch.zeros(V, dtype=torch.float32, device=dev)
    if method == "yu13":
        mean = torch.zeros((n, 3), device=dev)
        smoothed = torch.zeros((n, 3), device=dev)
        L.launchCalculationOfMeanAndSmoothParticles(*dims(n), prm, grid(parts), grid(mean), grid(smoothed), gC, spi)
        out["mean"], out["smoothed"] = mean.cpu().numpy(), smoothed.cpu().numpy()
        ninv_scan = torch.zeros(C, dtype=u32, device=dev)
        ni = L.launchThrustExclusivePrefixSumScan(ninv_scan.data_ptr(), ninv.data_ptr(), C)
        nb = L.launchThrustExclusivePrefixSumScan(band_scan.data_ptr(), band.data_ptr(), V)
        sv = torch.zeros(max(nb, 1), dtype=u32, device=dev)
        inv = torch.zeros(max(ni, 1), dtype=u32, device=dev)
        L.launchCompactationOfSurfaceVerticesAndParticles(*dims(max(C, V)), prm, grid(band, sc.resolution),
                                                          grid(band_scan, sc.resolution), grid(ninv, sp.resolution),
                                                          grid(ninv_scan, sp.resolution), gC,
                                                          GridT(sv.data_ptr(), nb, nb, uint3(nb, 1, 1)),
                                                          GridT(inv.data_ptr(), ni, ni, uint3(ni, 1, 1)))
        mats = torch.zeros((max(ni, 1), 9), device=dev)
        L.launchCalculationOfTransformMatricesForParticles(*dims(ni), prm, spi, grid(mean), grid(parts), gC,
                                                           GridT(inv.data_ptr(), ni, ni, uint3(ni, 1, 1)),
                                                           GridT(mats.data_ptr(), ni, ni, uint3(ni, 1, 1)))
        out["inv"], out["G"] = inv[:ni].cpu().numpy().view(np.uint32), mats[:ni].cpu().numpy()
        field.view(torch.int32).fill_(0x64646464)
        L.launchComputationOfScalarFieldGrid(*dims(nb), prm, nb, sci, spi,
                                             GridT(mats.data_ptr(), ni, ni, uint3(ni, 1, 1)), grid(smoothed),
                                             grid(dens), gC, GridT(sv.data_ptr(), nb, nb, uint3(nb, 1, 1)),
                                             grid(ninv, sp.resolution), grid(ninv_scan, sp.resolution),
                                             grid(field, sc.resolution))
    else:
        nb = L.launchThrustExclusivePrefixSumScan(band_scan.data_ptr(), band.data_ptr(), V)
        sv = torch.zeros(max(nb, 1), dtype=u32, device=dev)
        L.launchCompactSurfaceVertex(*dims(V), GridT(sv.data_ptr(), nb, nb, uint3(nb, 1, 1)),
                                     grid(band_scan, sc.resolution), grid(band, sc.resolution), prm)
        L.launchUpdateScalarGridValuesCompacted(*dims(nb), GridT(sv.data_ptr(), nb, nb, uint3(nb, 1, 1)), nb, gC,
                                                grid(parts), grid(field, sc.resolution), spi, sci, prm)
    out["sv"] = sv[:nb].cpu().numpy().view(np.uint32)
    out["phi"] = field.cpu().numpy()
    gsv = GridT(sv.data_ptr(), nb, nb, uint3(nb, 1, 1))
    valid = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    gvalid = GridT(valid.data_ptr(), nb, nb, uint3(nb, 1, 1))
    if method == "akinci":
        L.launchDetectionOfValidSurfaceCubesForAkinci(*dims(nb), gsv, nb, grid(field, sc.resolution), gvalid,
                                                      grid(band, sc.resolution), prm)
        out["valid"] = valid[:nb].cpu().numpy().view(np.uint32)
        return out
    nv = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    L.launchDetectValidSurfaceCubes(*dims(nb), gsv, nb, grid(field, sc.resolution), gvalid,
                                    GridT(nv.data_ptr(), nb, nb, uint3(nb, 1, 1)), grid(band, sc.resolution), prm)
    out["valid"] = valid[:nb].cpu().numpy().view(np.uint32)
    out["nverts"] = nv[:nb].cpu().numpy().view(np.uint32)
    vscan = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    nvscan = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    nq = L.launchThrustExclusivePrefixSumScan(vscan.data_ptr(), valid.data_ptr(), nb)
    nm = L.launchThrustExclusivePrefixSumScan(nvscan.data_ptr(), nv.data_ptr(), nb)
    vidx = torch.zeros(max(nq, 1), dtype=u32, device=dev)
    L.launchCompactValidSurfaceCubes(*dims(nb), GridT(vidx.data_ptr(), nq, nq, uint3(nq, 1, 1)),
                                     GridT(vscan.data_ptr(), nb, nb, uint3(nb, 1, 1)), gvalid, prm)
    mp = torch.zeros((max(nm, 1), 3), device=dev)
    mn = torch.zeros((max(nm, 1), 3), device=dev)
    L.launchGenerateTriangles(*dims(nq), gsv, GridT(vidx.data_ptr(), nq, nq, uint3(nq, 1, 1)), sci,
                              GridT(nvscan.data_ptr(), nb, nb, uint3(nb, 1, 1)), grid(field, sc.resolution),
                              GridT(mp.data_ptr(), nm, nm, uint3(nm, 1, 1)), GridT(mn.data_ptr(), nm, nm, uint3(nm, 1, 1)),
                              prm)
    out["mesh_pos"], out["mesh_nrm"] = mp[:nm].cpu().numpy(), mn[:nm].cpu().numpy()
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
