"""The reference's frame flow over its kernel-level ABI.  TEST INFRASTRUCTURE.

Restates the host side of the reference's per-frame loop
(ReconstructorGPU.cpp:25-79 and :292-313, ReconstructorGPUOurs.cpp:164-265,
ReconstructorGPUOursZB05.cpp:22-78 and :230-339, ReconstructorGPUOursYu13.cpp:
24-63 and :104-284, ReconstructorGPUAkinci12.cpp:34-84): the same launch*
calls in the same order, with the same buffers, memsets and launch shapes
(calcGridDimBlockDim, CudaUtils.h:87-106).  The launch* entry points come
from one of two libraries:

* ``"compat"``: this project's compatibility layer inside libfsr_gb300.so
  (csrc/compat.cu), whose kernels are its own;
* ``"reference"``: oracle/_build/libref_gpu.so, which launches the
  reference's own kernels from oracle/_ref/ref_kernels_sm103a.cubin
  (oracle/ref_gpu/ref_launchers.cu, oracle/ref_gpu/build_ref_gpu.sh).

``frame`` runs one frame and returns its outputs and the wall time of the
reference's timer scope: spatial hashing plus the frame's stages
(ReconstructorGPU.cpp:46-54; the launchers synchronise the device after
every kernel, so the wall time is the device time plus the launch gaps).
The buffers the reference allocates inside that scope are allocated there
too, through PyTorch's caching allocator (cheaper than the reference's
cudaMalloc/cudaFree: the difference favours the reference).  Two hazards of
the reference's kernels are guarded: the particle, mean and smoothed arrays
get one element more than the particle count, because
calculationOfMeanAndSmoothParticles (ReconstructionCUDA.cu:609, ``>``
instead of ``>=``) reads and writes index N; and the particles must lie in
the grid (calcParticlesHashKernel has no bounds check, cu:1391-1395).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
CUBIN = os.path.join(ORACLE, "_ref", "ref_kernels_sm103a.cubin")
REF_LIB = os.path.join(ORACLE, "_build", "libref_gpu.so")

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


def grid(t, res=None, n=None):
    """Grid<T> view of a tensor: a 3D grid when res is given, else a 1D array
    of n elements (default: rows of 3 floats count as one element each)."""
    if res is not None:
        n = res[0] * res[1] * res[2]
        r = uint3(*res)
    else:
        if n is None:
            n = t.shape[0] if (t.dim() >= 2 and t.shape[-1] == 3) else t.numel()
        r = uint3(n, 1, 1)
    return GridT(t.data_ptr(), n, n, r)


def ginfo(o):
    g = GridInfoC()
    g.minPos = float3(*o.minPos)
    g.maxPos = float3(*o.maxPos)
    g.cellSize = o.cellSize
    g.resolution = uint3(*o.res)
    return g


def available(which: str) -> bool:
    if which == "reference":
        return os.path.exists(CUBIN) and os.path.exists(REF_LIB)
    return True


_BOUND = {}


def launchers(which: str):
    """A proxy whose methods are the launch* entry points of `which`
    ("compat" or "reference"), taking the structs by reference."""
    if which in _BOUND:
        return _BOUND[which]
    if which == "reference":
        if not available("reference"):
            raise FileNotFoundError("the reference's kernels are not built (oracle/ref_gpu/build_ref_gpu.sh)")
        lib_path = REF_LIB
        ref = ctypes.CDLL(lib_path)
        ref.ref_gpu_load.restype = ctypes.c_int
        ref.ref_gpu_last_error.restype = ctypes.c_char_p
        if ref.ref_gpu_load(CUBIN.encode()) != 0:
            raise RuntimeError(ref.ref_gpu_last_error().decode())
    else:
        from fluidsurfacereconstructiongpu_gb300 import _native  # noqa: F401  (builds and loads the library)
        from fluidsurfacereconstructiongpu_gb300.build import LIB_PATH as lib_path
        ref = None
    out_dir = os.path.join(ORACLE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, f"libcompat_driver_{which}.so")
    src = os.path.join(HERE, "compat_driver.cpp")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(lib_path)):
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-o", so, src, "-I",
                        os.path.join(ROOT, "include"), "-I", cuda_inc, lib_path,
                        "-Wl,-rpath," + os.path.dirname(lib_path)], check=True)
    drv = ctypes.CDLL(so)
    drv.w_launchThrustExclusivePrefixSumScan.restype = c_uint
    drv.w_launchThrustExclusivePrefixSumScan.argtypes = [c_vp, c_vp, c_uint]

    class Proxy:
        def last_error(self):
            return ref.ref_gpu_last_error().decode() if ref is not None else ""

        def __getattr__(self, name):
            f = getattr(drv, "w_" + name)
            if name == "launchThrustExclusivePrefixSumScan":
                return f

            def call(*args):
                conv = [ctypes.byref(a) if isinstance(a, ctypes.Structure) else a for a in args]
                return f(*conv)
            return call
    _BOUND[which] = Proxy()
    return _BOUND[which]


_TABLES = {}


def bind_tables(L, dev="cuda"):
    """Uploads the marching-cubes tables in the reference's layout and binds
    them (bindTextures, ReconstructionCUDA.cu:49-65, as the reference's
    initialisation does)."""
    import torch
    from oracle import pipeline as P
    if "t" not in _TABLES:
        lib = P.load("oracle32")
        e = np.zeros(256, np.uint32)
        t = np.zeros(256 * 16, np.int32)
        n = np.zeros(256, np.uint32)
        c = np.zeros(24, np.uint32)
        lib.o_mc_reference_tables(P._ptr(e), P._ptr(t), P._ptr(n), P._ptr(c))
        _TABLES["t"] = [torch.from_numpy(a.view(np.int32)).to(dev) for a in (e, t, n, c)]
    d = _TABLES["t"]
    L.bindTextures(c_vp(d[0].data_ptr()), c_vp(d[1].data_ptr()), c_vp(d[2].data_ptr()), c_vp(d[3].data_ptr()))


def frame(L, method, fr, params, outputs=True):
    """One frame of `method` through the launchers L.  Returns (outputs,
    seconds of the reference's timer scope); outputs holds the stage results
    as numpy arrays when `outputs` is set, else only the sizes."""
    import torch
    from oracle import pipeline as P
    prm = params.simparam()
    iso, ratio, scale, _ = params.resolved()
    sp, sc = P.grid_derive(fr.bbox_min, fr.bbox_max, fr.h, scale, ratio)
    spi, sci = ginfo(sp), ginfo(sc)
    C, V, n = sp.count, sc.count, fr.n
    dev = "cuda"
    u32 = torch.int32
    # beginFrame / onBeginFrame (outside the timer): upload and per-frame grids
    pos_np = np.concatenate([fr.pos, fr.pos[-1:]]) if n else np.zeros((1, 3), np.float32)
    parts = torch.from_numpy(np.ascontiguousarray(pos_np)).to(dev)  # n + 1 rows (cu:609)
    dens = torch.from_numpy(np.ascontiguousarray(fr.density)).to(dev)
    sflag = torch.zeros(n, dtype=u32, device=dev)
    field = torch.zeros(V, dtype=torch.float32, device=dev)
    band = torch.zeros(V, dtype=u32, device=dev)
    band_scan = torch.zeros(V, dtype=u32, device=dev)
    if method == "yu13":
        ninv = torch.zeros(C, dtype=u32, device=dev)
        ninv_scan = torch.zeros(C, dtype=u32, device=dev)
        mean = torch.zeros((n + 1, 3), device=dev)
        smoothed = torch.zeros((n + 1, 3), device=dev)
    torch.cuda.synchronize()
    out = {}
    t0 = time.perf_counter()

    # spatialHashingGridBuilding (ReconstructorGPU.cpp:292-313)
    flag = torch.zeros(C, dtype=torch.float32, device=dev)
    ranges = torch.empty((C, 2), dtype=u32, device=dev).fill_(-1)
    gparts = grid(parts, n=n)
    L.launchSpatialGridBuilding(gparts, grid(dens), n, grid(ranges, sp.resolution), grid(flag, sp.resolution), spi)
    gC = grid(ranges, sp.resolution)

    # surface particles
    if method == "yu13":
        sflag.zero_()
        ninv.zero_()
        L.launchExtractionOfSurfaceAndInvolveParticles(*dims(C), prm, grid(flag, sp.resolution),
                                                       grid(ninv, sp.resolution), grid(sflag), gC)
    elif method == "akinci":
        L.launchExtractionOfSurfaceParticlesForAkinci(*dims(n), prm, gparts, grid(dens), gC, spi, grid(sflag))
    else:
        sflag.zero_()
        L.launchExtractionOfSurfaceParticles(*dims(C), prm, grid(flag, sp.resolution), grid(sflag), gC)
    # band
    band.zero_()
    L.launchEstimationOfSurfaceVertices(*dims(n), prm, sci, gparts, grid(sflag), gC, grid(band, sc.resolution))

    if method == "yu13":
        L.launchCalculationOfMeanAndSmoothParticles(*dims(n), prm, gparts, grid(mean, n=n), grid(smoothed, n=n),
                                                    gC, spi)
        ni = L.launchThrustExclusivePrefixSumScan(ninv_scan.data_ptr(), ninv.data_ptr(), C)
        nb = L.launchThrustExclusivePrefixSumScan(band_scan.data_ptr(), band.data_ptr(), V)
        if ni == 0 or nb == 0:  # the reference stops the frame here (Yu13.cpp:178-188)
            raise ValueError("frame without involved particles or band vertices")
        sv = torch.zeros(max(nb, 1), dtype=u32, device=dev)
        inv = torch.zeros(max(ni, 1), dtype=u32, device=dev)
        gsv = GridT(sv.data_ptr(), nb, nb, uint3(nb, 1, 1))
        ginv = GridT(inv.data_ptr(), ni, ni, uint3(ni, 1, 1))
        L.launchCompactationOfSurfaceVerticesAndParticles(*dims(max(C, V)), prm, grid(band, sc.resolution),
                                                          grid(band_scan, sc.resolution), grid(ninv, sp.resolution),
                                                          grid(ninv_scan, sp.resolution), gC, gsv, ginv)
        mats = torch.zeros((max(ni, 1), 9), device=dev)
        gmats = GridT(mats.data_ptr(), ni, ni, uint3(ni, 1, 1))
        L.launchCalculationOfTransformMatricesForParticles(*dims(ni), prm, spi, grid(mean, n=n), gparts, gC, ginv,
                                                           gmats)
        field.view(torch.int32).fill_(0x64646464)  # cudaMemset(..., 100, ...), Yu13.cpp:264
        L.launchComputationOfScalarFieldGrid(*dims(nb), prm, nb, sci, spi, gmats, grid(smoothed, n=n), grid(dens),
                                             gC, gsv, grid(ninv, sp.resolution), grid(ninv_scan, sp.resolution),
                                             grid(field, sc.resolution))
    else:
        nb = L.launchThrustExclusivePrefixSumScan(band_scan.data_ptr(), band.data_ptr(), V)
        if nb == 0:  # the reference stops the frame here (ZB05.cpp:275-279)
            raise ValueError("frame without band vertices")
        sv = torch.zeros(max(nb, 1), dtype=u32, device=dev)
        gsv = GridT(sv.data_ptr(), nb, nb, uint3(nb, 1, 1))
        L.launchCompactSurfaceVertex(*dims(V), gsv, grid(band_scan, sc.resolution), grid(band, sc.resolution), prm)
        field.zero_()
        L.launchUpdateScalarGridValuesCompacted(*dims(nb), gsv, nb, gC, gparts, grid(field, sc.resolution), spi, sci,
                                                prm)
    valid = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    gvalid = GridT(valid.data_ptr(), nb, nb, uint3(nb, 1, 1))
    if method == "akinci":
        L.launchDetectionOfValidSurfaceCubesForAkinci(*dims(nb), gsv, nb, grid(field, sc.resolution), gvalid,
                                                      grid(band, sc.resolution), prm)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out.update(n_band=nb)
        if outputs:
            out.update(pos=parts[:n].cpu().numpy(), ranges=ranges.cpu().numpy().view(np.uint32),
                       sflag=sflag.cpu().numpy().view(np.uint32), is_surf=band.cpu().numpy().view(np.uint32),
                       sv=sv[:nb].cpu().numpy().view(np.uint32), phi=field.cpu().numpy(),
                       valid=valid[:nb].cpu().numpy().view(np.uint32))
        return out, dt
    nv = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    L.launchDetectValidSurfaceCubes(*dims(nb), gsv, nb, grid(field, sc.resolution), gvalid,
                                    GridT(nv.data_ptr(), nb, nb, uint3(nb, 1, 1)), grid(band, sc.resolution), prm)
    vscan = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    nvscan = torch.zeros(max(nb, 1), dtype=u32, device=dev)
    nq = L.launchThrustExclusivePrefixSumScan(vscan.data_ptr(), valid.data_ptr(), nb)
    nm = L.launchThrustExclusivePrefixSumScan(nvscan.data_ptr(), nv.data_ptr(), nb)
    if nm == 0:  # ReconstructorGPUOurs.cpp:205-209
        raise ValueError("frame without mesh vertices")
    vidx = torch.zeros(max(nq, 1), dtype=u32, device=dev)
    L.launchCompactValidSurfaceCubes(*dims(nb), GridT(vidx.data_ptr(), nq, nq, uint3(nq, 1, 1)),
                                     GridT(vscan.data_ptr(), nb, nb, uint3(nb, 1, 1)), gvalid, prm)
    mp = torch.zeros((max(nm, 1), 3), device=dev)
    mn = torch.zeros((max(nm, 1), 3), device=dev)
    L.launchGenerateTriangles(*dims(nq), gsv, GridT(vidx.data_ptr(), nq, nq, uint3(nq, 1, 1)), sci,
                              GridT(nvscan.data_ptr(), nb, nb, uint3(nb, 1, 1)), grid(field, sc.resolution),
                              GridT(mp.data_ptr(), nm, nm, uint3(nm, 1, 1)), GridT(mn.data_ptr(), nm, nm, uint3(nm, 1, 1)),
                              prm)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    out.update(n_band=nb, n_valid=nq, n_mesh_vertices=nm)
    if outputs:
        out.update(pos=parts[:n].cpu().numpy(), ranges=ranges.cpu().numpy().view(np.uint32),
                   sflag=sflag.cpu().numpy().view(np.uint32), is_surf=band.cpu().numpy().view(np.uint32),
                   sv=sv[:nb].cpu().numpy().view(np.uint32), phi=field.cpu().numpy(),
                   valid=valid[:nb].cpu().numpy().view(np.uint32), nverts=nv[:nb].cpu().numpy().view(np.uint32),
                   mesh_pos=mp[:nm].cpu().numpy(), mesh_nrm=mn[:nm].cpu().numpy())
        if method == "yu13":
            out.update(ninv=ninv.cpu().numpy().view(np.uint32), mean=mean[:n].cpu().numpy(),
                       smoothed=smoothed[:n].cpu().numpy(), inv=inv[:ni].cpu().numpy().view(np.uint32),
                       G=mats[:ni].cpu().numpy())
    return out, dt
