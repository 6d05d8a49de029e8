"""Python front end over the C ABI (include/fsr.h).

Two layers:

* :class:`Reconstructor` - one handle, one frame per call, particles either
  as CUDA tensors (device path, ``fsr_reconstruct``) or numpy arrays (host
  path, ``fsr_reconstruct_host``);
* the reference-named file-driven classes ``ReconstructorGPUOursZB05``,
  ``ReconstructorGPUOursYu13``, ``ReconstructorGPUAkinci12`` (and a TC01
  variant) with the public methods of ReconstructorGPU
  (FluidSurfaceReconstruction/GPU/ReconstructorGPU.h:14-30).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native as N

METHODS = {"zb05": N.METHOD_ZB05, "tc01": N.METHOD_TC01, "yu13": N.METHOD_YU13, "aniso": N.METHOD_YU13,
           "akinci": N.METHOD_AKINCI12, "akinci12": N.METHOD_AKINCI12}


def header_from(bbox_min, bbox_max, h, particle_radius, mass) -> N.FrameHeader:
    hd = N.FrameHeader()
    for a in range(3):
        hd.bbox_min[a] = float(bbox_min[a])
        hd.bbox_max[a] = float(bbox_max[a])
    hd.kernel_radius = float(h)
    hd.particle_radius = float(particle_radius)
    hd.particle_mass = float(mass)
    return hd


def header_of(frame) -> N.FrameHeader:
    """Header of a synthetic ParticleFrame (or anything with the same fields)."""
    return header_from(frame.bbox_min, frame.bbox_max, frame.h, frame.particle_radius, frame.mass)


def default_params(method: str) -> N.Params:
    p = N.Params()
    N.check(N.lib.fsr_default_params(METHODS[method], ctypes.byref(p)))
    return p


@dataclass
class Mesh:
    positions: np.ndarray  # (3T, 3) f32, triangle soup in the reference's order
    normals: np.ndarray

    @property
    def n_triangles(self) -> int:
        return self.positions.shape[0] // 3


@dataclass
class IndexedMesh:
    positions: np.ndarray  # (V, 3) f32, shared vertices in order of first use
    normals: np.ndarray
    triangles: np.ndarray  # (T, 3) u32 vertex indices, the soup's triangle order


class Reconstructor:
    """One reconstructor handle bound to a CUDA device."""

    def __init__(self, method: str = "zb05", device: int = 0, *, iso: Optional[float] = None,
                 grid_ratio: Optional[int] = None, cell_size_scale: Optional[float] = None,
                 smoothing_lambda: Optional[float] = None, aniso_radius_over_h: Optional[float] = None,
                 min_neighbors: Optional[int] = None, keep_intermediates: bool = False,
                 stage_timing: bool = False, weld: bool = False, compute_density: bool = False):
        self.method = method
        p = default_params(method)
        if iso is not None:
            p.iso_value = iso
        if grid_ratio is not None:
            p.grid_ratio = grid_ratio
        if cell_size_scale is not None:
            p.cell_size_scale = cell_size_scale
        if smoothing_lambda is not None:
            p.smoothing_lambda = smoothing_lambda
        if aniso_radius_over_h is not None:
            p.aniso_radius_over_h = aniso_radius_over_h
        if min_neighbors is not None:
            p.min_neighbors = min_neighbors
        p.flags = (N.FLAG_KEEP_INTERMEDIATES if keep_intermediates else 0) | \
            (N.FLAG_STAGE_TIMING if stage_timing else 0) | (N.FLAG_WELD if weld else 0) | \
            (N.FLAG_COMPUTE_DENSITY if compute_density else 0)
        self.params = p
        h = ctypes.c_void_p()
        st = N.lib.fsr_create(ctypes.byref(p), int(device), ctypes.byref(h))
        if st != N.FSR_OK:
            raise N.FsrError(st, "fsr_create failed")
        self._h = h

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            N.lib.fsr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- frames
    def reconstruct(self, xyz, density, header: N.FrameHeader, stream=None) -> int:
        """Device path: xyz (N,3) and density (N,) float32 CUDA tensors
        (density may be None with compute_density=True).  Returns the number
        of mesh vertices; the mesh stays on the device."""
        import torch
        assert xyz.is_cuda and (density is None or density.is_cuda), "device path needs CUDA tensors"
        xyz = xyz.contiguous()
        assert xyz.dtype == torch.float32
        n = int(xyz.numel() // 3)
        dptr = None
        if density is not None:
            density = density.contiguous()
            assert density.dtype == torch.float32 and int(density.numel()) == n
            dptr = density.data_ptr()
        s = stream if stream is not None else torch.cuda.current_stream(xyz.device)
        st = N.lib.fsr_reconstruct(self._h, ctypes.byref(header), ctypes.c_void_p(xyz.data_ptr()),
                                   ctypes.c_void_p(dptr), n, ctypes.c_void_p(s.cuda_stream))
        N.check(st, self._h)
        return int(self.stats().n_mesh_vertices)

    def reconstruct_host(self, xyz: np.ndarray, density: np.ndarray, header: N.FrameHeader,
                         capacity: Optional[int] = None) -> Mesh:
        """Host path: numpy in, numpy triangle soup out (copies included)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        density = np.ascontiguousarray(density, dtype=np.float32).reshape(-1)
        nv = ctypes.c_uint64(0)
        cap = int(capacity) if capacity is not None else 0
        pos = np.empty((max(cap, 1), 3), np.float32)
        nrm = np.empty((max(cap, 1), 3), np.float32)
        st = N.lib.fsr_reconstruct_host(self._h, ctypes.byref(header), xyz.ctypes.data, density.ctypes.data,
                                        xyz.shape[0], pos.ctypes.data, nrm.ctypes.data, cap, ctypes.byref(nv),
                                        None)
        if st == 7:  # capacity: fetch with the right size
            pos = np.empty((nv.value, 3), np.float32)
            nrm = np.empty((nv.value, 3), np.float32)
            N.check(N.lib.fsr_copy_mesh(self._h, pos.ctypes.data, nrm.ctypes.data, nv.value, ctypes.byref(nv)),
                    self._h)
            return Mesh(pos, nrm)
        N.check(st, self._h)
        return Mesh(pos[:nv.value], nrm[:nv.value])

    def reconstruct_host_frames(self, frames, capacity: Optional[int] = None, stream=None):
        """A sequence of frames, host memory in and out, with each frame's
        upload and read-back overlapped with its neighbours' reconstruction
        (fsr_reconstruct_host_frames).  `frames`: (xyz, density, header)
        triples.  Returns one Mesh per frame; raises on the first failing
        frame.  `capacity` (mesh vertices per frame) defaults to a bound from
        the grid: pass the expected size to keep the pinned outputs small."""
        import torch
        ins, outs = [], []
        arr = (N.HostFrame * len(frames))()
        for k, (xyz, density, header) in enumerate(frames):
            xyz = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)).pin_memory()
            den = torch.from_numpy(np.ascontiguousarray(density, dtype=np.float32).reshape(-1)).pin_memory()
            n = xyz.shape[0]
            cap = int(capacity) if capacity is not None else max(4096, 24 * n)
            pos = torch.empty((cap, 3), dtype=torch.float32).pin_memory()
            nrm = torch.empty((cap, 3), dtype=torch.float32).pin_memory()
            ins.append((xyz, den))
            outs.append((pos, nrm))
            arr[k].header = header
            arr[k].xyz = xyz.data_ptr()
            arr[k].density = den.data_ptr()
            arr[k].n = n
            arr[k].out_pos = pos.data_ptr()
            arr[k].out_nrm = nrm.data_ptr()
            arr[k].capacity = cap
        st = N.lib.fsr_reconstruct_host_frames(self._h, arr, len(frames),
                                               None if stream is None else ctypes.c_void_p(stream))
        if st not in (0, 7):
            N.check(st, self._h)
        out = []
        for k in range(len(frames)):
            nv = arr[k].n_vertices
            if arr[k].status == 7:  # outputs too small: this frame again on its own, sized by the call
                xyz, den = ins[k]
                out.append(self.reconstruct_host(xyz.numpy(), den.numpy(), frames[k][2]))
            else:
                N.check(arr[k].status, self._h)
                out.append(Mesh(outs[k][0][:nv].numpy().copy(), outs[k][1][:nv].numpy().copy()))
        if st == 7 and arr[len(frames) - 1].status == 0:  # the handle holds the last frame again
            xyz, den = ins[-1]
            self.reconstruct_host(xyz.numpy(), den.numpy(), frames[-1][2])
        return out

    def mesh(self) -> Mesh:
        nv = int(self.stats().n_mesh_vertices)
        pos = np.empty((max(nv, 1), 3), np.float32)
        nrm = np.empty((max(nv, 1), 3), np.float32)
        out = ctypes.c_uint64(0)
        N.check(N.lib.fsr_copy_mesh(self._h, pos.ctypes.data, nrm.ctypes.data, nv, ctypes.byref(out)), self._h)
        return Mesh(pos[:nv], nrm[:nv])

    def mesh_tensors(self, stream=None):
        """The last frame's triangle soup as two (3T, 3) CUDA tensors (copies)."""
        import torch
        nv = int(self.stats().n_mesh_vertices)
        pos = torch.empty((nv, 3), dtype=torch.float32, device="cuda")
        nrm = torch.empty((nv, 3), dtype=torch.float32, device="cuda")
        s = stream if stream is not None else torch.cuda.current_stream()
        out = ctypes.c_uint64(0)
        N.check(N.lib.fsr_copy_mesh_device(self._h, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(nrm.data_ptr()),
                                           nv, ctypes.byref(out), ctypes.c_void_p(s.cuda_stream)), self._h)
        return pos, nrm

    def backward(self, grad_mesh_pos, stream=None, with_radius: bool = False):
        """dL/d(particle positions) (N, 3) in input order from dL/d(mesh vertex
        positions) (3T, 3) of the last frame; optionally also dL/d(particle
        radius) (ZB05 / Akinci12)."""
        import torch
        n = int(self.stats().n_particles)
        g = grad_mesh_pos.contiguous().to(torch.float32)
        assert g.is_cuda and g.shape == (int(self.stats().n_mesh_vertices), 3)
        out = torch.empty((n, 3), dtype=torch.float32, device=g.device)
        s = stream if stream is not None else torch.cuda.current_stream(g.device)
        rad = ctypes.c_float(0.0)
        N.check(N.lib.fsr_backward(self._h, ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                   ctypes.byref(rad) if with_radius else None, ctypes.c_void_p(s.cuda_stream)),
                self._h)
        return (out, float(rad.value)) if with_radius else out

    def mesh_device_ptrs(self):
        p, q, nv = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_uint64()
        N.check(N.lib.fsr_mesh_device(self._h, ctypes.byref(p), ctypes.byref(q), ctypes.byref(nv)), self._h)
        return p.value, q.value, nv.value

    def pair_counts(self, stream=None) -> dict:
        """Candidate and contributing pairs of the last frame's neighbour-sum
        stages (fsr_count_pairs); synchronises the stream."""
        import torch
        pc = N.PairCounts()
        s = stream if stream is not None else torch.cuda.current_stream()
        N.check(N.lib.fsr_count_pairs(self._h, ctypes.byref(pc), ctypes.c_void_p(s.cuda_stream)), self._h)
        return {name: int(getattr(pc, name)) for name, _ in N.PairCounts._fields_}

    def stats(self) -> N.Stats:
        s = N.Stats()
        N.check(N.lib.fsr_get_stats(self._h, ctypes.byref(s)), self._h)
        return s

    def write_vis(self, path: str, mesh_name: str) -> None:
        """The last frame's intermediates as a .vis file (the reference
        viewer's debug dump); mesh_name is recorded as its mesh file."""
        N.check(N.lib.fsr_write_vis(self._h, path.encode(), mesh_name.encode()), self._h)

    def indexed_mesh(self) -> "IndexedMesh":
        """The last frame's welded mesh (needs weld=True)."""
        s = self.stats()
        nv, ni = int(s.n_weld_vertices), int(s.n_mesh_vertices)
        pos = np.empty((nv, 3), np.float32)
        nrm = np.empty((nv, 3), np.float32)
        idx = np.empty(ni, np.uint32)
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        N.check(N.lib.fsr_copy_indexed_mesh(self._h, pos.ctypes.data, nrm.ctypes.data, nv, idx.ctypes.data, ni,
                                            ctypes.byref(a), ctypes.byref(b)), self._h)
        return IndexedMesh(pos, nrm, idx.reshape(-1, 3))

    def debug(self, name: str) -> np.ndarray:
        which = N.DBG[name]
        need = ctypes.c_uint64(0)
        N.check(N.lib.fsr_debug_fetch(self._h, which, None, 0, ctypes.byref(need)), self._h)
        if name == "weld_keys":
            out = np.empty(need.value // 8, dtype=np.uint64)
            if need.value:
                N.check(N.lib.fsr_debug_fetch(self._h, which, out.ctypes.data, need.value, None), self._h)
            return out
        dtype = np.float32 if name in ("sorted_xyz", "field", "mean", "smoothed", "G", "density") else np.uint32
        out = np.empty(need.value // 4, dtype=dtype)
        if need.value:
            N.check(N.lib.fsr_debug_fetch(self._h, which, out.ctypes.data, need.value, None), self._h)
        if name in ("sorted_xyz", "mean", "smoothed"):
            out = out.reshape(-1, 3)
        elif name == "ranges":
            out = out.reshape(-1, 2)
        elif name == "G":
            out = out.reshape(-1, 9)
        return out


class Batch:
    """Many frames (mixed methods, uneven sizes) in one CUDA graph launch.

    ``params`` maps method names to keyword overrides of that method's
    defaults (the Reconstructor keywords iso, grid_ratio, cell_size_scale,
    smoothing_lambda, aniso_radius_over_h, min_neighbors)."""

    def __init__(self, device: int = 0, params: Optional[dict] = None):
        arr = (N.Params * 4)()
        for m in range(4):
            N.check(N.lib.fsr_default_params(m, ctypes.byref(arr[m])))
        for name, kw in (params or {}).items():
            p = arr[METHODS[name]]
            for k, v in kw.items():
                setattr(p, "iso_value" if k == "iso" else k, v)
        self._arr = arr
        h = ctypes.c_void_p()
        N.check(N.lib.fsr_batch_create(arr, int(device), ctypes.byref(h)))
        self._b = h
        self.count = 0

    def close(self):
        if getattr(self, "_b", None):
            N.lib.fsr_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != N.FSR_OK:
            raise N.FsrError(st, N.lib.fsr_batch_last_error(self._b).decode())

    def reconstruct(self, frames, stream=None, retune: bool = False, autotune: bool = True):
        """frames: list of (method, xyz (N,3) float32, density (N,), header);
        xyz/density CUDA tensors or numpy arrays."""
        import torch
        arr = (N.BatchFrame * len(frames))()
        keep = []
        for i, (method, xyz, den, hdr) in enumerate(frames):
            if isinstance(xyz, np.ndarray):
                xyz = np.ascontiguousarray(xyz, np.float32)
                den = np.ascontiguousarray(den, np.float32)
                px, pd = xyz.ctypes.data, den.ctypes.data
            else:
                xyz = xyz.contiguous()
                den = den.contiguous()
                px, pd = xyz.data_ptr(), den.data_ptr()
            keep.append((xyz, den))
            arr[i].header = hdr
            arr[i].method = METHODS[method]
            arr[i].n_particles = int(den.shape[0])
            arr[i].xyz = px
            arr[i].density = pd
        flags = (N.BATCH_RETUNE if retune else 0) | (0 if autotune else N.BATCH_NO_AUTOTUNE)
        s = stream if stream is not None else torch.cuda.current_stream()
        self._check(N.lib.fsr_reconstruct_batch(self._b, arr, len(frames), flags, ctypes.c_void_p(s.cuda_stream)))
        self.count = len(frames)

    def tuning(self) -> N.BatchTuning:
        t = N.BatchTuning()
        self._check(N.lib.fsr_batch_get_tuning(self._b, ctypes.byref(t)))
        return t

    def stats(self, i: int) -> N.Stats:
        st = N.Stats()
        self._check(N.lib.fsr_batch_frame_stats(self._b, i, ctypes.byref(st)))
        return st

    def mesh(self, i: int) -> Mesh:
        nv = int(self.stats(i).n_mesh_vertices)
        pos = np.empty((max(nv, 1), 3), np.float32)
        nrm = np.empty((max(nv, 1), 3), np.float32)
        out = ctypes.c_uint64(0)
        self._check(N.lib.fsr_batch_copy_mesh(self._b, i, pos.ctypes.data, nrm.ctypes.data, nv, ctypes.byref(out)))
        return Mesh(pos[:nv], nrm[:nv])


def set_io_threads(n: int) -> None:
    """Host threads of the .xyz reader and .obj writer (0: one per core)."""
    N.lib.fsr_io_set_threads(int(n))


def read_xyz(path: str):
    """Parses an .xyz file; returns (header, xyz (N,3), density (N,))."""
    return _read_particles(N.lib.fsr_read_xyz, path)


def read_xyz_binary(path: str):
    """Reads an .xyzb sidecar; returns (header, xyz (N,3), density (N,))."""
    return _read_particles(N.lib.fsr_read_xyz_binary, path)


def write_xyz_binary(path: str, header, xyz, density) -> None:
    """Writes particles as an .xyzb file (the binary form of an .xyz)."""
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    den = np.ascontiguousarray(density, np.float32).reshape(-1)
    if den.shape[0] != xyz.shape[0]:
        raise ValueError("xyz and density differ in length")
    N.check(N.lib.fsr_write_xyz_binary(path.encode(), ctypes.byref(header), xyz.ctypes.data, den.ctypes.data,
                                       xyz.shape[0]))


def _read_particles(fn, path: str):
    hd = N.FrameHeader()
    px, pd, n = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_uint64()
    N.check(fn(path.encode(), ctypes.byref(hd), ctypes.byref(px), ctypes.byref(pd), ctypes.byref(n)))
    try:
        cnt = n.value
        xyz = np.ctypeslib.as_array((ctypes.c_float * (3 * max(cnt, 1))).from_address(px.value))[:3 * cnt]
        den = np.ctypeslib.as_array((ctypes.c_float * max(cnt, 1)).from_address(pd.value))[:cnt]
        xyz = xyz.reshape(-1, 3).copy()
        den = den.copy()
    finally:
        N.lib.fsr_free_host(px)
        N.lib.fsr_free_host(pd)
    return hd, xyz, den


def write_xyz(path: str, frame) -> None:
    """Writes a ParticleFrame as .xyz (data_format.txt layout)."""
    with open(path, "w") as f:
        f.write("%.9g %.9g %.9g\n" % tuple(frame.bbox_min))
        f.write("%.9g %.9g %.9g\n" % tuple(frame.bbox_max))
        f.write("%.9g\n%.9g\n%.9g\n" % (frame.h, frame.particle_radius, frame.mass))
        for p, d in zip(frame.pos, frame.density):
            f.write("%.9g %.9g %.9g %.9g\n" % (p[0], p[1], p[2], d))


def write_obj(path: str, mesh) -> None:
    """Writes a Mesh (triangle soup) or an IndexedMesh as .obj."""
    pos = np.ascontiguousarray(mesh.positions, np.float32)
    nrm = np.ascontiguousarray(mesh.normals, np.float32)
    if isinstance(mesh, IndexedMesh):
        idx = np.ascontiguousarray(mesh.triangles, np.uint32).reshape(-1)
        N.check(N.lib.fsr_write_obj_indexed(path.encode(), pos.ctypes.data, nrm.ctypes.data, pos.shape[0],
                                            idx.ctypes.data, idx.shape[0]))
        return
    N.check(N.lib.fsr_write_obj(path.encode(), pos.ctypes.data, nrm.ctypes.data, pos.shape[0]))


class ReconstructorGPU:
    """File-driven reconstruction with the reference's public interface
    (ReconstructorGPU.h:14-30): frames [from, to) of
    directory + pattern % frame + '.xyz', meshes to the same stem + '.obj'."""

    METHOD = "zb05"
    ALGORITHM = ""

    def __init__(self, directory: str, file_pattern: str, frame_from: int, frame_to: int, device: int = 0,
                 **params):
        self.directory = directory
        self.file_pattern = file_pattern
        self.frame_from, self.frame_to = int(frame_from), int(frame_to)
        self._save_obj = True
        self._save_cfg = False
        self._rec = Reconstructor(self.METHOD, device, **params)
        self._times: list[float] = []
        self._num_particles = 0
        self._sidecar = False
        self._indexed = False
        self._save_vis = False
        self._io = None

    def getAlgorithmType(self) -> str:
        return self.ALGORITHM

    def setOutputMeshFile(self, flag: bool):
        self._save_obj = bool(flag)

    def setOutputConfigFile(self, flag: bool):
        self._save_cfg = bool(flag)

    def setOutputVisualizeFile(self, flag: bool):
        self._save_vis = bool(flag)

    def setIndexedMesh(self, flag: bool):
        """Write welded (indexed) .obj files instead of triangle soups."""
        self._indexed = bool(flag)
        p = self._rec.params
        p.flags = (p.flags | N.FLAG_WELD) if flag else (p.flags & ~N.FLAG_WELD)
        N.check(N.lib.fsr_set_params(self._rec._h, ctypes.byref(p)), self._rec._h)

    def setBinarySidecar(self, flag: bool):
        """Read stem.xyzb instead of parsing stem.xyz when it is current, and
        write it after parsing (FSR_FILES_SIDECAR)."""
        self._sidecar = bool(flag)

    def ioTiming(self):
        """Host timings of the last reconstruct() (fsr_files_timing)."""
        return self._io

    def getSimulationParameters(self) -> N.Params:
        return self._rec.params

    def getNumberOfParticles(self) -> int:
        return int(self._rec.stats().n_particles) if self._times else 0

    def getTimeConsumingSequence(self) -> list:
        return list(self._times)

    def reconstruct(self):
        if self.frame_from >= self.frame_to:
            raise ValueError("Wrong settings occur for frame range.")
        n = self.frame_to - self.frame_from
        ms = (ctypes.c_double * n)()
        d = self.directory if self.directory.endswith(os.sep) or not self.directory else self.directory + os.sep
        flags = (N.FILES_WRITE_OBJ if self._save_obj else 0) | (N.FILES_SIDECAR if self._sidecar else 0) | \
            (N.FILES_INDEXED_OBJ if self._indexed else 0) | (N.FILES_WRITE_VIS if self._save_vis else 0)
        tm = N.FilesTiming()
        st = N.lib.fsr_reconstruct_files_ex(self._rec._h, d.encode(), self.file_pattern.encode(),
                                            self.frame_from, self.frame_to, flags, ms, ctypes.byref(tm))
        N.check(st, self._rec._h)
        self._io = tm
        self._times = list(ms)
        if self._save_cfg:
            s = self._rec.stats()
            with open(os.path.join(d, self.ALGORITHM + ".config"), "w") as f:
                f.write(f"{s.n_mesh_vertices // 3}\n{s.n_surface_particles / max(s.n_particles, 1)}\n"
                        f"{s.n_band_vertices / max(s.n_grid_vertices, 1)}\n")
        with open(os.path.join(d, self.ALGORITHM + ".time"), "a") as f:
            f.write(" ".join("%g" % t for t in self._times) + " \n")


class ReconstructorGPUOursZB05(ReconstructorGPU):
    METHOD = "zb05"
    ALGORITHM = "Our Algorithm using ZB05 kernel"


class ReconstructorGPUOursTC01(ReconstructorGPU):
    METHOD = "tc01"
    ALGORITHM = "Our Algorithm using TC01 kernel"


class ReconstructorGPUOursYu13(ReconstructorGPU):
    METHOD = "yu13"
    ALGORITHM = "Our Algorithm using anisotropic kernel"


class ReconstructorGPUAkinci12(ReconstructorGPU):
    METHOD = "akinci"
    ALGORITHM = "Akinci12 using ZB05 kernel"
