"""Composition of the oracle stages into whole frames.  TEST INFRASTRUCTURE.

Mirrors the reference's per-frame stage order on its dense layouts:

* ``zb05`` / ``tc01``: ReconstructorGPUOursZB05.cpp:22-78 (TC01 swaps the
  field function, ReconstructionCUDA.cu:178-227, which has no caller there);
* ``yu13``: ReconstructorGPUOursYu13.cpp:24-63;
* ``akinci``: ReconstructorGPUAkinci12.cpp:34-84 (host marching cubes).

Spatial hashing follows ReconstructionCUDA.cu:1437-1481: the stable
``sort_by_key`` is numpy's stable argsort and the cell ranges are the segment
bounds of the sorted keys; the thrust exclusive scans are numpy cumulative
sums.  Those three results are defined exactly, so any correct
implementation gives the same integers.

The stage library is one of

* ``liboracle32`` - this project's FP32 restatement (oracle/fsr_oracle.c),
* ``liboracle64`` - the same with FP64 continuous values,
* ``libfsr_refkernels`` - the reference's own kernels compiled for the host
  (oracle/build_ref.sh), present only where the reference sources were.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EMPTY = np.uint32(0xFFFFFFFF)
YU13_FILL_BITS = np.uint32(0x64646464)  # memset(…, 100, …), ReconstructorGPUOursYu13.cpp:264


class SimParam(ctypes.Structure):
    """Layout of SimParam (Defines.h:18-32)."""

    _fields_ = [
        ("particleRadius", ctypes.c_float),
        ("particleMass", ctypes.c_float),
        ("smoothingRadius", ctypes.c_float),
        ("smoothingRadiusSq", ctypes.c_float),
        ("smoothingRadiusInv", ctypes.c_float),
        ("lambdaForSmoothed", ctypes.c_float),
        ("anisotropicRadius", ctypes.c_float),
        ("isoValue", ctypes.c_float),
        ("scSpGridResRatio", ctypes.c_uint32),
        ("expandExtent", ctypes.c_uint32),
        ("minNumNeighbors", ctypes.c_uint32),
        ("spatialCellSizeScale", ctypes.c_float),
    ]


class GridInfo(ctypes.Structure):
    """Layout of GridInfo (Defines.h:62-68)."""

    _fields_ = [
        ("minPos", ctypes.c_float * 3),
        ("maxPos", ctypes.c_float * 3),
        ("cellSize", ctypes.c_float),
        ("res", ctypes.c_uint32 * 3),
    ]

    @property
    def resolution(self):
        return (int(self.res[0]), int(self.res[1]), int(self.res[2]))

    @property
    def count(self):
        r = self.resolution
        return r[0] * r[1] * r[2]


# Reference defaults per method (onInitialization of each reconstructor).
METHOD_DEFAULTS = {
    # ReconstructorGPUOursZB05.cpp:85-97
    "zb05": dict(iso=-0.0001, ratio=2, cell_scale=1.0, expand=4),
    "tc01": dict(iso=0.25, ratio=2, cell_scale=1.0, expand=4),
    # ReconstructorGPUOursYu13.cpp:78-99, anisotropic radius 2h at :21
    "yu13": dict(iso=0.0, ratio=3, cell_scale=1.3, expand=3, lam=0.5, min_neighbors=25,
                 aniso_radius_over_h=2.0),
    # ReconstructorGPUAkinci12.cpp:93-106
    "akinci": dict(iso=-0.0001, ratio=2, cell_scale=1.0, expand=4),
}


@dataclass
class FrameParams:
    """Per-frame parameters: the .xyz header plus the reconstructor settings."""

    method: str
    h: float
    particle_radius: float
    mass: float
    iso: Optional[float] = None
    ratio: Optional[int] = None
    cell_scale: Optional[float] = None
    lam: float = 0.5
    aniso_radius: Optional[float] = None  # absolute; default 2h
    min_neighbors: int = 25

    def resolved(self):
        d = METHOD_DEFAULTS[self.method]
        iso = d["iso"] if self.iso is None else self.iso
        ratio = d["ratio"] if self.ratio is None else self.ratio
        scale = d["cell_scale"] if self.cell_scale is None else self.cell_scale
        ar = (2.0 * self.h) if self.aniso_radius is None else self.aniso_radius
        return iso, int(ratio), float(scale), float(ar)

    def simparam(self) -> SimParam:
        iso, ratio, scale, ar = self.resolved()
        h = np.float32(self.h)
        p = SimParam()
        p.particleRadius = np.float32(self.particle_radius)
        p.particleMass = np.float32(self.mass)
        p.smoothingRadius = h
        p.smoothingRadiusSq = np.float32(h * h)
        p.smoothingRadiusInv = np.float32(1.0 / np.float64(h))  # 1.0 / h in double, ReconstructorGPU.cpp:237
        p.lambdaForSmoothed = np.float32(self.lam)
        # anisotropicRadius = h * 2 in FP32 (Yu13.cpp:21) unless given
        p.anisotropicRadius = np.float32(h * np.float32(2)) if self.aniso_radius is None else np.float32(ar)
        p.isoValue = np.float32(iso)
        p.scSpGridResRatio = ratio
        p.expandExtent = METHOD_DEFAULTS[self.method]["expand"]
        p.minNumNeighbors = int(self.min_neighbors)
        p.spatialCellSizeScale = np.float32(scale)
        return p


_LIBS = {}


def _ptr(a: Optional[np.ndarray]):
    if a is None:
        return ctypes.c_void_p(0)
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the oracle must be contiguous"
    return ctypes.c_void_p(a.ctypes.data)


def lib_path(kind: str) -> str:
    if kind == "oracle32":
        return os.path.join(HERE, "_build", "liboracle32.so")
    if kind == "oracle64":
        return os.path.join(HERE, "_build", "liboracle64.so")
    if kind == "ref":
        return os.path.join(HERE, "_ref", "libfsr_refkernels.so")
    raise ValueError(kind)


def available(kind: str) -> bool:
    return os.path.exists(lib_path(kind))


def load(kind: str):
    if kind in _LIBS:
        return _LIBS[kind]
    path = lib_path(kind)
    if not os.path.exists(path):
        raise FileNotFoundError(f"{kind} stage library not built: {path}")
    lib = ctypes.CDLL(path)
    lib.o_mc_cpu.restype = ctypes.c_int64
    if hasattr(lib, "o_mc_cpu2"):
        lib.o_mc_cpu2.restype = ctypes.c_int64
    _LIBS[kind] = lib
    return lib


def set_threads(kind: str, n: int) -> int:
    return int(load(kind).o_set_threads(int(n)))


def grid_derive(bbmin, bbmax, h, cell_scale, ratio):
    """Spatial and scalar grids of ReconstructorGPU.cpp:237-268 and :99-105."""
    lib = load("oracle32")
    sp, sc = GridInfo(), GridInfo()
    bmin = np.ascontiguousarray(bbmin, dtype=np.float32)
    bmax = np.ascontiguousarray(bbmax, dtype=np.float32)
    rc = lib.o_grid_derive(_ptr(bmin), _ptr(bmax), ctypes.c_float(h), ctypes.c_float(cell_scale),
                           ctypes.c_uint32(ratio), ctypes.byref(sp), ctypes.byref(sc))
    if rc != 0:
        raise ValueError("invalid grid parameters")
    return sp, sc


def cell_ranges(sorted_keys: np.ndarray, n_cells: int) -> np.ndarray:
    """[start, end) of every cell in the sorted key array, 0xFFFFFFFF if empty
    (findCellRangeKernel, ReconstructionCUDA.cu:1399-1435)."""
    ranges = np.full((n_cells, 2), EMPTY, dtype=np.uint32)
    if sorted_keys.size == 0:
        return ranges
    change = np.flatnonzero(np.diff(sorted_keys)) + 1
    starts = np.concatenate(([0], change)).astype(np.uint32)
    ends = np.concatenate((change, [sorted_keys.size])).astype(np.uint32)
    k = sorted_keys[starts]
    ranges[k, 0] = starts
    ranges[k, 1] = ends
    return ranges


def exclusive_scan(a: np.ndarray) -> tuple[np.ndarray, int]:
    """thrust::exclusive_scan plus the total (ReconstructionCUDA.cu:1154-1172)."""
    if a.size == 0:
        return a.astype(np.uint32), 0
    c = np.cumsum(a, dtype=np.uint64)
    total = int(c[-1])
    out = np.empty(a.size, dtype=np.uint32)
    out[0] = 0
    out[1:] = (c[:-1] & 0xFFFFFFFF).astype(np.uint32)
    return out, total


@dataclass
class Frame:
    """Every intermediate of one frame, in the reference's layouts."""

    method: str
    spatial: GridInfo
    scalar: GridInfo
    simparam: SimParam
    keys: np.ndarray = None          # unsorted cell id per input particle
    perm: np.ndarray = None          # stable sort permutation
    pos: np.ndarray = None           # sorted positions (N,3) f32
    dens: np.ndarray = None          # sorted densities (N,) f32
    flag: np.ndarray = None          # occupancy (C,) f32
    ranges: np.ndarray = None        # (C,2) u32
    sflag: np.ndarray = None         # surface particle flags (N,) u32
    ninv: Optional[np.ndarray] = None
    is_surf: np.ndarray = None       # dense band flags (V,) u32
    sv: np.ndarray = None            # band vertex ids (B,) u32
    mean: Optional[np.ndarray] = None
    mean32: Optional[np.ndarray] = None
    smoothed: Optional[np.ndarray] = None
    inv: Optional[np.ndarray] = None
    G: Optional[np.ndarray] = None
    phi: np.ndarray = None           # dense field (V,) real
    valid: np.ndarray = None         # (B,) u32
    nverts: Optional[np.ndarray] = None
    valid_idx: np.ndarray = None     # positions in sv of valid cubes (Q,)
    nv_scan: Optional[np.ndarray] = None
    mesh_pos: np.ndarray = None      # (3T,3) real
    mesh_nrm: np.ndarray = None
    extra: dict = field(default_factory=dict)

    @property
    def n_triangles(self) -> int:
        return 0 if self.mesh_pos is None else self.mesh_pos.shape[0] // 3


class _TimedLib:
    """Wraps a stage library and accumulates wall time per o_* call."""

    def __init__(self, lib, times: dict):
        self._lib, self._t = lib, times

    def __getattr__(self, name):
        f = getattr(self._lib, name)
        if not name.startswith("o_") or name in ("o_real_bytes", "o_is_reference"):
            return f

        def call(*a):
            import time
            t0 = time.perf_counter()
            r = f(*a)
            self._t[name] = self._t.get(name, 0.0) + time.perf_counter() - t0
            return r
        return call


def run_frame(kind: str, pos_in: np.ndarray, dens_in: np.ndarray, bbmin, bbmax,
              params: FrameParams, times: Optional[dict] = None, field_stride: int = 1) -> Frame:
    """Runs one frame of ``params.method`` with stage library ``kind``.

    times: if given, receives the wall seconds spent in each stage library
    call.  field_stride > 1 evaluates the field only at every field_stride-th
    band vertex (a bounded timing sample: the field call's time is then
    scaled by the sampling factor and the mesh is not meaningful)."""
    lib = load(kind)
    if times is not None:
        lib = _TimedLib(lib, times)
    real = np.float64 if lib.o_real_bytes() == 8 else np.float32
    is_ref = bool(lib.o_is_reference())
    iso, ratio, scale, _ = params.resolved()
    sp, sc = grid_derive(bbmin, bbmax, params.h, scale, ratio)
    prm = params.simparam()
    fr = Frame(method=params.method, spatial=sp, scalar=sc, simparam=prm)
    C, V = sp.count, sc.count
    pos_in = np.ascontiguousarray(pos_in, dtype=np.float32).reshape(-1, 3)
    dens_in = np.ascontiguousarray(dens_in, dtype=np.float32).reshape(-1)
    n = pos_in.shape[0]

    # --- spatial hashing (ReconstructorGPU.cpp:292-313, cu:1437-1481)
    keys = np.zeros(n, dtype=np.uint32)
    flag = np.zeros(C, dtype=np.float32)
    rc = lib.o_hash(_ptr(pos_in), ctypes.c_uint32(n), ctypes.byref(sp), _ptr(keys), _ptr(flag))
    if rc != 0:
        raise ValueError("particle outside the spatial grid")
    perm = np.argsort(keys, kind="stable").astype(np.uint32)
    skeys = keys[perm]
    pos = np.ascontiguousarray(pos_in[perm])
    dens = np.ascontiguousarray(dens_in[perm])
    ranges = cell_ranges(skeys, C)
    fr.keys, fr.perm, fr.pos, fr.dens, fr.flag, fr.ranges = keys, perm, pos, dens, flag, ranges

    # --- surface particles
    sflag = np.zeros(n, dtype=np.uint32)
    if params.method == "yu13":
        ninv = np.zeros(C, dtype=np.uint32)
        lib.o_surface_involve(ctypes.byref(prm), _ptr(flag), _ptr(ranges), ctypes.byref(sp),
                              _ptr(sflag), ctypes.c_uint32(n), _ptr(ninv))
        fr.ninv = ninv
    elif params.method == "akinci":
        lib.o_colorfield(ctypes.byref(prm), _ptr(pos), _ptr(dens), ctypes.c_uint32(n), _ptr(ranges),
                         ctypes.byref(sp), _ptr(sflag))
    else:
        lib.o_surface(ctypes.byref(prm), _ptr(flag), _ptr(ranges), ctypes.byref(sp), _ptr(sflag),
                      ctypes.c_uint32(n))
    fr.sflag = sflag

    # --- narrow band
    is_surf = np.zeros(V, dtype=np.uint32)
    lib.o_band(ctypes.byref(prm), ctypes.byref(sc), _ptr(pos), _ptr(sflag), ctypes.c_uint32(n),
               _ptr(ranges), ctypes.byref(sp), _ptr(is_surf))
    sv = np.flatnonzero(is_surf == 1).astype(np.uint32)
    nb = sv.size
    fr.is_surf, fr.sv = is_surf, sv

    # --- field
    if params.method == "yu13":
        mean = np.zeros((n, 3), dtype=real)
        smoothed = np.zeros((n, 3), dtype=real)
        if is_ref:
            lib.o_smooth(ctypes.byref(prm), _ptr(pos), ctypes.c_uint32(n), _ptr(ranges),
                         ctypes.byref(sp), _ptr(mean), _ptr(smoothed))
            mean32 = mean
        else:
            mean32 = np.zeros((n, 3), dtype=np.float32)
            lib.o_smooth2(ctypes.byref(prm), _ptr(pos), ctypes.c_uint32(n), _ptr(ranges),
                          ctypes.byref(sp), _ptr(mean32), _ptr(mean), _ptr(smoothed))
        ninv = fr.ninv
        ninv_scan, ni = exclusive_scan(ninv)
        cells = np.flatnonzero(ninv > 0)
        if ni:
            starts = ranges[cells, 0].astype(np.int64)
            counts = (ranges[cells, 1] - ranges[cells, 0]).astype(np.int64)
            inv = (np.repeat(starts - np.concatenate(([0], np.cumsum(counts)[:-1])), counts)
                   + np.arange(int(counts.sum()))).astype(np.uint32)
        else:
            inv = np.zeros(0, dtype=np.uint32)
        G = np.zeros((max(ni, 1), 9), dtype=real)
        if is_ref:
            lib.o_cov(ctypes.byref(prm), ctypes.byref(sp), _ptr(mean), _ptr(pos), ctypes.c_uint32(n),
                      _ptr(ranges), _ptr(inv), ctypes.c_uint32(ni), _ptr(G))
        else:
            lib.o_cov2(ctypes.byref(prm), ctypes.byref(sp), _ptr(mean32), _ptr(mean), _ptr(pos),
                       ctypes.c_uint32(n), _ptr(ranges), _ptr(inv), ctypes.c_uint32(ni), _ptr(G))
        G = G[:ni]
        phi = np.full(V, YU13_FILL_BITS, dtype=np.uint32).view(np.float32).astype(real)
        svf = np.ascontiguousarray(sv[::field_stride]) if field_stride > 1 else sv
        t_before = times.get("o_field_aniso", 0.0) if times is not None else 0.0
        lib.o_field_aniso(ctypes.byref(prm), ctypes.c_uint32(svf.size), ctypes.byref(sc), ctypes.byref(sp),
                          _ptr(np.ascontiguousarray(G) if ni else np.zeros((1, 9), dtype=real)),
                          ctypes.c_uint32(ni), _ptr(smoothed), _ptr(dens), ctypes.c_uint32(n),
                          _ptr(ranges), _ptr(svf), _ptr(ninv), _ptr(ninv_scan), _ptr(phi))
        if times is not None and svf.size:
            dt = times["o_field_aniso"] - t_before
            times["o_field_aniso"] = t_before + dt * nb / svf.size
            times["_unsampled_extra"] = times.get("_unsampled_extra", 0.0) + dt * (nb / svf.size - 1.0)
        fr.mean, fr.mean32, fr.smoothed, fr.inv, fr.G = mean, mean32, smoothed, inv, G
        fr.extra["ninv_scan"] = ninv_scan
    else:
        phi = np.zeros(V, dtype=real)
        name = "o_field_tc01" if params.method == "tc01" else "o_field_zb05"
        svf = np.ascontiguousarray(sv[::field_stride]) if field_stride > 1 else sv
        t_before = times.get(name, 0.0) if times is not None else 0.0
        getattr(lib, name)(_ptr(svf), ctypes.c_uint32(svf.size), _ptr(ranges), _ptr(pos), ctypes.c_uint32(n),
                           ctypes.byref(sp), ctypes.byref(sc), ctypes.byref(prm), _ptr(phi))
        if times is not None and svf.size:
            dt = times[name] - t_before
            times[name] = t_before + dt * nb / svf.size
            times["_unsampled_extra"] = times.get("_unsampled_extra", 0.0) + dt * (nb / svf.size - 1.0)
    fr.phi = phi

    # --- marching cubes
    _marching_cubes(lib, fr, phi, real)
    return fr


def _marching_cubes(lib, fr: Frame, phi: np.ndarray, real, with_lengths: bool = False) -> None:
    """Marching-cubes stages on the frame's band and the given dense field
    (ReconstructorGPUOurs.cpp:164-265; Akinci12.cpp:213-288)."""
    sv, is_surf, prm, sc = fr.sv, fr.is_surf, fr.simparam, fr.scalar
    nb = sv.size
    valid = np.zeros(nb, dtype=np.uint32)
    if fr.method == "akinci":
        lib.o_classify_akinci(_ptr(sv), ctypes.c_uint32(nb), _ptr(phi), ctypes.byref(sc),
                              _ptr(is_surf), ctypes.byref(prm), _ptr(valid))
        valid_idx = np.flatnonzero(valid == 1).astype(np.uint32)
        cube_vertex = np.ascontiguousarray(sv[valid_idx])
        cap = 15 * valid_idx.size
        mp = np.zeros((max(cap, 1), 3), dtype=real)
        mn = np.zeros((max(cap, 1), 3), dtype=real)
        if with_lengths:
            ln = np.zeros(max(cap, 1), dtype=real)
            cnt = lib.o_mc_cpu2(_ptr(phi), ctypes.byref(sc), ctypes.c_float(prm.isoValue), _ptr(cube_vertex),
                                ctypes.c_uint32(valid_idx.size), _ptr(mp), _ptr(mn), _ptr(ln),
                                ctypes.c_uint64(cap))
        else:
            cnt = lib.o_mc_cpu(_ptr(phi), ctypes.byref(sc), ctypes.c_float(prm.isoValue), _ptr(cube_vertex),
                               ctypes.c_uint32(valid_idx.size), _ptr(mp), _ptr(mn), ctypes.c_uint64(cap))
        if cnt < 0:
            raise RuntimeError("host marching cubes overflow")
        fr.valid, fr.valid_idx = valid, valid_idx
        fr.mesh_pos, fr.mesh_nrm = mp[:cnt], mn[:cnt]
        if with_lengths:
            fr.extra["normal_len"] = ln[:cnt]
        return
    nverts = np.zeros(nb, dtype=np.uint32)
    lib.o_classify(_ptr(sv), ctypes.c_uint32(nb), _ptr(phi), ctypes.byref(sc), _ptr(is_surf),
                   ctypes.byref(prm), _ptr(valid), _ptr(nverts))
    valid_idx = np.flatnonzero(valid == 1).astype(np.uint32)
    nv_scan, total = exclusive_scan(nverts)
    mp = np.zeros((max(total, 1), 3), dtype=real)
    mn = np.zeros((max(total, 1), 3), dtype=real)
    if with_lengths:
        ln = np.zeros(max(total, 1), dtype=real)
        lib.o_generate2(_ptr(sv), ctypes.c_uint32(nb), _ptr(valid_idx), ctypes.c_uint32(valid_idx.size),
                        ctypes.byref(sc), _ptr(nv_scan), _ptr(phi), ctypes.byref(prm), _ptr(mp), _ptr(mn),
                        _ptr(ln), ctypes.c_uint64(total))
        fr.extra["normal_len"] = ln[:total]
    else:
        lib.o_generate(_ptr(sv), ctypes.c_uint32(nb), _ptr(valid_idx), ctypes.c_uint32(valid_idx.size),
                       ctypes.byref(sc), _ptr(nv_scan), _ptr(phi), ctypes.byref(prm), _ptr(mp), _ptr(mn),
                       ctypes.c_uint64(total))
    fr.valid, fr.nverts, fr.valid_idx, fr.nv_scan = valid, nverts, valid_idx, nv_scan
    fr.mesh_pos, fr.mesh_nrm = mp[:total], mn[:total]


def marching_cubes_on(kind: str, fr: Frame, band_values: np.ndarray) -> Frame:
    """Re-runs only the marching-cubes stages of a frame with library `kind`
    on a field given at the frame's band vertices (e.g. a GPU's field); the
    rest of the grid keeps the method's fill value.  Returns a new Frame
    sharing the frame's inputs."""
    lib = load(kind)
    real = np.float64 if lib.o_real_bytes() == 8 else np.float32
    if fr.method == "yu13":
        phi = np.full(fr.scalar.count, YU13_FILL_BITS, dtype=np.uint32).view(np.float32).astype(real)
    else:
        phi = np.zeros(fr.scalar.count, dtype=real)
    phi[fr.sv] = np.asarray(band_values, dtype=np.float32).astype(real)
    out = Frame(method=fr.method, spatial=fr.spatial, scalar=fr.scalar, simparam=fr.simparam)
    out.sv, out.is_surf, out.phi = fr.sv, fr.is_surf, phi
    _marching_cubes(lib, out, phi, real, with_lengths=True)
    return out


def cube_cases(kind: str, fr: Frame, cubes: np.ndarray) -> np.ndarray:
    """MC case index of each listed cube origin, from the frame's field."""
    lib = load(kind)
    out = np.zeros(cubes.size, dtype=np.uint32)
    c = np.ascontiguousarray(cubes, dtype=np.uint32)
    lib.o_cases(_ptr(c), ctypes.c_uint32(c.size), _ptr(fr.phi), ctypes.byref(fr.scalar),
                ctypes.byref(fr.simparam), _ptr(out))
    return out


def sph_density(pos: np.ndarray, h: float, mass: float) -> np.ndarray:
    """FP64 SPH density of every particle: m sigma / h^3 sum_j (1 - r_ij^2 /
    h^2)^3 over the particles within h (i itself included), sigma = 315 /
    (64 pi), the normalisation of the reference's field kernel (anisotropicW,
    ReconstructionCUDA.cuh:294-310, at G = I / h).  The reference has no
    density pass of its own (its .xyz files carry densities); this is the
    checker of the library's FSR_FLAG_COMPUTE_DENSITY.  All pairs, in blocks
    (for test-sized inputs)."""
    p = np.asarray(pos, np.float64).reshape(-1, 3)
    h = float(np.float32(h))
    h2 = h * h
    out = np.zeros(p.shape[0])
    blk = 2048
    for a in range(0, p.shape[0], blk):
        d = p[a:a + blk, None, :] - p[None, :, :]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        u = np.where(r2 < h2, 1.0 - r2 / h2, 0.0)
        out[a:a + blk] = (u * u * u).sum(axis=1)
    sigma = 315.0 / (64.0 * np.pi)
    return float(np.float32(mass)) * sigma / h ** 3 * out
