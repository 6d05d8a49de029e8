"""ctypes binding of libfsr_gb300.so (include/fsr.h).

The library is the only compute path: if it is missing or cannot be loaded
the import of this module raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB_PATH

c_u32 = ctypes.c_uint32
c_u64 = ctypes.c_uint64
c_f32 = ctypes.c_float
c_vp = ctypes.c_void_p

FSR_OK = 0
STATUS_NAMES = {
    0: "FSR_OK", 1: "FSR_ERR_INVALID_ARGUMENT", 2: "FSR_ERR_OUT_OF_GRID", 3: "FSR_ERR_CUDA",
    4: "FSR_ERR_OUT_OF_MEMORY", 5: "FSR_ERR_IO", 6: "FSR_ERR_FORMAT", 7: "FSR_ERR_CAPACITY",
    8: "FSR_ERR_TOO_LARGE", 9: "FSR_ERR_NOT_READY",
}

METHOD_ZB05, METHOD_TC01, METHOD_YU13, METHOD_AKINCI12 = 0, 1, 2, 3
FLAG_KEEP_INTERMEDIATES = 0x1
FLAG_STAGE_TIMING = 0x2
FLAG_SMALL_POOLS = 0x4
FLAG_WELD = 0x8
FLAG_COMPUTE_DENSITY = 0x10

DBG = dict(perm=0, sorted_xyz=1, ranges=2, surface_flags=3, involved_counts=4, band=5, field=6,
           mc_info=7, valid=8, mean=9, smoothed=10, G=11, weld_keys=12, density=13)

NUM_STAGES = 12
STAGE_NAMES = ["hash+sort", "ranges", "surface", "band stamp", "band list", "smoothing", "covariance",
               "field", "mc classify", "mc scans", "mc generate", "readback"]


class Params(ctypes.Structure):
    _fields_ = [("method", c_u32), ("iso_value", c_f32), ("grid_ratio", c_u32), ("cell_size_scale", c_f32),
                ("smoothing_lambda", c_f32), ("aniso_radius_over_h", c_f32), ("min_neighbors", c_u32),
                ("flags", c_u32)]


class FrameHeader(ctypes.Structure):
    _fields_ = [("bbox_min", c_f32 * 3), ("bbox_max", c_f32 * 3), ("kernel_radius", c_f32),
                ("particle_radius", c_f32), ("particle_mass", c_f32)]


class HostFrame(ctypes.Structure):
    _fields_ = [("header", FrameHeader), ("xyz", c_vp), ("density", c_vp), ("n", c_u64), ("out_pos", c_vp),
                ("out_nrm", c_vp), ("capacity", c_u64), ("n_vertices", c_u64), ("status", ctypes.c_int)]


class PairCounts(ctypes.Structure):
    _fields_ = [("smooth_candidates", c_u64), ("smooth_contributing", c_u64), ("cov_candidates", c_u64),
                ("cov_contributing", c_u64), ("field_candidates", c_u64), ("field_contributing", c_u64),
                ("color_candidates", c_u64), ("color_contributing", c_u64)]


class Stats(ctypes.Structure):
    _fields_ = [("n_particles", c_u64), ("n_cells", c_u64), ("n_grid_vertices", c_u64),
                ("n_surface_particles", c_u64), ("n_involved_particles", c_u64), ("n_band_vertices", c_u64),
                ("n_valid_cubes", c_u64), ("n_mesh_vertices", c_u64), ("spatial_res", c_u32 * 3),
                ("scalar_res", c_u32 * 3), ("n_fp64_fallbacks", c_u32), ("n_retries", c_u32),
                ("n_kernel_launches", c_u32), ("n_backward_launches", c_u32),
                ("stage_ms", c_f32 * NUM_STAGES), ("total_ms", c_f32), ("device_bytes", c_u64),
                ("n_weld_vertices", c_u64)]


class FsrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class BatchFrame(ctypes.Structure):
    _fields_ = [("header", FrameHeader), ("method", c_u32), ("reserved", c_u32), ("n_particles", c_u64),
                ("xyz", c_vp), ("density", c_vp)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("lanes", c_u32), ("grid_div", c_u32), ("n_candidates", c_u32), ("kernels_per_launch", c_u32),
                ("graph_ms", c_f32), ("frames_ms", c_f32), ("block_threads", c_u32)]


BATCH_RETUNE = 0x1
BATCH_NO_AUTOTUNE = 0x2

FILES_WRITE_OBJ = 0x1
FILES_SIDECAR = 0x2
FILES_INDEXED_OBJ = 0x4
FILES_WRITE_VIS = 0x8


class FilesTiming(ctypes.Structure):
    _fields_ = [("read_ms", ctypes.c_double), ("upload_ms", ctypes.c_double), ("reconstruct_ms", ctypes.c_double),
                ("write_ms", ctypes.c_double), ("wall_ms", ctypes.c_double)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libfsr_gb300.so is not built ({LIB_PATH}); run __graft_entry__.build()")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    sig = {
        "fsr_abi_version": (c_u32, []),
        "fsr_build_info": (ctypes.c_char_p, []),
        "fsr_default_params": (ctypes.c_int, [c_u32, P(Params)]),
        "fsr_create": (ctypes.c_int, [P(Params), ctypes.c_int, P(c_vp)]),
        "fsr_destroy": (None, [c_vp]),
        "fsr_set_params": (ctypes.c_int, [c_vp, P(Params)]),
        "fsr_last_error": (ctypes.c_char_p, [c_vp]),
        "fsr_reconstruct": (ctypes.c_int, [c_vp, P(FrameHeader), c_vp, c_vp, c_u64, c_vp]),
        "fsr_reconstruct_host": (ctypes.c_int, [c_vp, P(FrameHeader), c_vp, c_vp, c_u64, c_vp, c_vp, c_u64,
                                                P(c_u64), c_vp]),
        "fsr_reconstruct_host_frames": (ctypes.c_int, [c_vp, P(HostFrame), c_u32, c_vp]),
        "fsr_mesh_device": (ctypes.c_int, [c_vp, P(c_vp), P(c_vp), P(c_u64)]),
        "fsr_copy_mesh": (ctypes.c_int, [c_vp, c_vp, c_vp, c_u64, P(c_u64)]),
        "fsr_get_stats": (ctypes.c_int, [c_vp, P(Stats)]),
        "fsr_copy_mesh_device": (ctypes.c_int, [c_vp, c_vp, c_vp, c_u64, P(c_u64), c_vp]),
        "fsr_backward": (ctypes.c_int, [c_vp, c_vp, c_vp, P(c_f32), c_vp]),
        "fsr_batch_create": (ctypes.c_int, [c_vp, ctypes.c_int, P(c_vp)]),
        "fsr_batch_destroy": (None, [c_vp]),
        "fsr_batch_last_error": (ctypes.c_char_p, [c_vp]),
        "fsr_reconstruct_batch": (ctypes.c_int, [c_vp, c_vp, c_u32, c_u32, c_vp]),
        "fsr_batch_get_tuning": (ctypes.c_int, [c_vp, P(BatchTuning)]),
        "fsr_batch_frame_stats": (ctypes.c_int, [c_vp, c_u32, P(Stats)]),
        "fsr_batch_mesh_device": (ctypes.c_int, [c_vp, c_u32, P(c_vp), P(c_vp), P(c_u64)]),
        "fsr_batch_copy_mesh": (ctypes.c_int, [c_vp, c_u32, c_vp, c_vp, c_u64, P(c_u64)]),
        "fsr_debug_fetch": (ctypes.c_int, [c_vp, c_u32, c_vp, c_u64, P(c_u64)]),
        "fsr_count_pairs": (ctypes.c_int, [c_vp, P(PairCounts), c_vp]),
        "fsr_measure_fp32_rate": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_double)]),
        "fsr_read_xyz": (ctypes.c_int, [ctypes.c_char_p, P(FrameHeader), P(c_vp), P(c_vp), P(c_u64)]),
        "fsr_free_host": (None, [c_vp]),
        "fsr_write_obj": (ctypes.c_int, [ctypes.c_char_p, c_vp, c_vp, c_u64]),
        "fsr_reconstruct_files": (ctypes.c_int, [c_vp, ctypes.c_char_p, ctypes.c_char_p, c_u32, c_u32,
                                                 ctypes.c_int, P(ctypes.c_double)]),
        "fsr_reconstruct_files_ex": (ctypes.c_int, [c_vp, ctypes.c_char_p, ctypes.c_char_p, c_u32, c_u32, c_u32,
                                                    P(ctypes.c_double), P(FilesTiming)]),
        "fsr_io_set_threads": (None, [c_u32]),
        "fsr_copy_indexed_mesh": (ctypes.c_int, [c_vp, c_vp, c_vp, c_u64, c_vp, c_u64, P(c_u64), P(c_u64)]),
        "fsr_write_obj_indexed": (ctypes.c_int, [ctypes.c_char_p, c_vp, c_vp, c_u64, c_vp, c_u64]),
        "fsr_write_vis": (ctypes.c_int, [c_vp, ctypes.c_char_p, ctypes.c_char_p]),
        "fsr_check_division": (ctypes.c_int, [c_f32, P(c_u64), P(c_u64)]),
        "fsr_check_spiky_grad": (ctypes.c_int, [ctypes.c_double, P(c_u64), P(c_u64)]),
        "fsr_write_xyz_binary": (ctypes.c_int, [ctypes.c_char_p, P(FrameHeader), c_vp, c_vp, c_u64]),
        "fsr_read_xyz_binary": (ctypes.c_int, [ctypes.c_char_p, P(FrameHeader), P(c_vp), P(c_vp), P(c_u64)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def check(status: int, handle=None):
    if status != FSR_OK:
        msg = lib.fsr_last_error(handle).decode() if handle else ""
        raise FsrError(status, msg)
