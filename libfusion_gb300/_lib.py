"""ctypes binding of the libgbfusion C ABI (include/gbfusion.h).

Loading fails loudly when the shared library has not been built: there is no
CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libgbfusion.so"

MAX_LEVELS = 5
OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "OUT_OF_MEMORY", 4: "CAPACITY", 5: "NO_DEVICE", 6: "IO"}

FLAG_POOL_EXHAUSTED = 1
FLAG_HASH_FULL = 2
FLAG_COORD_RANGE = 4
FLAG_TRACK_FAILED = 8
FLAG_NAN_POSE = 16

VOXEL_REF = 0
VOXEL_HALF = 1
VOXEL_SNORM = 2
MESH_VERTEX, MESH_NORMAL, MESH_COLOUR = 0, 1, 2


class Intrinsics(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float)]


class Config(C.Structure):
    _fields_ = [
        ("voxel_size", C.c_float), ("truncation", C.c_float),
        ("zmin_update", C.c_float), ("zmax_update", C.c_float),
        ("zmin_raycast", C.c_float), ("zmax_raycast", C.c_float),
        ("num_buckets", C.c_int32), ("num_blocks", C.c_int32), ("voxel_layout", C.c_int32),
        ("num_levels", C.c_int32), ("max_iterations", C.c_int32 * MAX_LEVELS),
        ("w_icp", C.c_float), ("w_rgb", C.c_float),
        ("icp_dist_thresh", C.c_float), ("icp_angle_thresh", C.c_float),
        ("bilateral", C.c_int32), ("max_probe", C.c_int32), ("motion_prior", C.c_int32),
    ]


class TrackResult(C.Structure):
    _fields_ = [("success", C.c_int32), ("iterations", C.c_int32), ("icp_error", C.c_float),
                ("rgb_error", C.c_float), ("icp_inliers", C.c_float), ("rgb_inliers", C.c_float),
                ("update", C.c_double * 16)]


class FrameStats(C.Structure):
    _fields_ = [("frame_index", C.c_int64), ("allocated_blocks", C.c_int32), ("visible_blocks", C.c_int32),
                ("render_blocks_valid", C.c_int32), ("status", C.c_uint32), ("track", TrackResult),
                ("level_iterations", C.c_int32 * MAX_LEVELS), ("pixel_iterations", C.c_int64),
                ("integrated_blocks", C.c_int64)]


class ReduceInputs(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float),
                ("ref_vmap", C.c_void_p), ("ref_nmap", C.c_void_p), ("ref_intensity", C.c_void_p),
                ("cur_vmap", C.c_void_p), ("cur_nmap", C.c_void_p), ("cur_intensity", C.c_void_p),
                ("cur_didx", C.c_void_p), ("cur_didy", C.c_void_p),
                ("dist_thresh", C.c_float), ("angle_thresh", C.c_float)]


class MapSize(C.Structure):
    """MapSize (include/data_struct/map_struct.h:53-58)."""
    _fields_ = [("num_blocks", C.c_int32), ("num_hash_entries", C.c_int32), ("num_buckets", C.c_int32)]


class SlotResult(C.Structure):
    _fields_ = [("pose", C.c_double * 16), ("tracked", C.c_int32), ("status", C.c_uint32),
                ("frame_index", C.c_int64)]


TUNE_MAX_REPORT = 16


class LaunchShape(C.Structure):
    _fields_ = [("groups", C.c_int32), ("stagger", C.c_int32), ("ray_tile_w", C.c_int32), ("median_ms", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("state", C.c_int32), ("from_table", C.c_int32), ("ticks_per_candidate", C.c_int32),
                ("chosen", LaunchShape), ("n_tried", C.c_int32), ("tried", LaunchShape * TUNE_MAX_REPORT)]


class SynthParams(C.Structure):
    _fields_ = [("room", C.c_float * 3), ("n_spheres", C.c_int32), ("n_boxes", C.c_int32),
                ("sphere_rmin", C.c_float), ("sphere_rmax", C.c_float), ("seed", C.c_uint64),
                ("trajectory", C.c_int32), ("radius", C.c_float), ("height", C.c_float),
                ("yaw_jitter_deg", C.c_float), ("speed", C.c_float), ("fps", C.c_float),
                ("frames_per_loop", C.c_int32), ("noise", C.c_float), ("zclip_min", C.c_float),
                ("zclip_max", C.c_float)]


_P = C.c_void_p
_I32, _I64, _U64 = C.c_int32, C.c_int64, C.c_uint64
_D16 = C.POINTER(C.c_double)

# name -> (restype, argtypes); every function declared with GBF_API in gbfusion.h
SIGNATURES = {
    "gbf_version": (C.c_char_p, []),
    "gbf_last_error": (C.c_char_p, []),
    "gbf_config_default": (C.c_int, [C.POINTER(Config)]),
    "gbf_session_bytes": (C.c_int, [C.POINTER(Config), C.POINTER(Intrinsics), C.POINTER(C.c_uint64)]),
    "gbf_session_create": (C.c_int, [C.POINTER(Config), C.POINTER(Intrinsics), C.POINTER(_P)]),
    "gbf_session_destroy": (C.c_int, [_P]),
    "gbf_session_reset": (C.c_int, [_P, _P]),
    "gbf_session_inputs": (C.c_int, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "gbf_session_stage": (C.c_int, [_P, _P, _I64, _P, _I64, _P]),
    "gbf_set_pose": (C.c_int, [_P, _D16, _P]),
    "gbf_get_pose": (C.c_int, [_P, _D16, _P]),
    "gbf_get_stats": (C.c_int, [_P, C.POINTER(FrameStats), _P]),
    "gbf_fuse": (C.c_int, [_P, _P, _I64, _P, _I64, _P, _I64, _D16, _P]),
    "gbf_raycast": (C.c_int, [_P, _D16, _P, _I64, _P]),
    "gbf_raycast_maps": (C.c_int, [_P, _D16, _P, _I64, _P, _I64, _P, _I64, _P]),
    "gbf_extract_mesh": (C.c_int, [_P, _I32, _P, _P, _U64, C.POINTER(C.c_uint64), _P]),
    "gbf_build_pyramid": (C.c_int, [_P, _I32, _P, _I64, _P, _I64, _P]),
    "gbf_reduce": (C.c_int, [_P, _I32, _D16, C.c_float, _D16, _P]),
    "gbf_reduce_noalloc": (C.c_int, [C.POINTER(ReduceInputs), _D16, C.c_float, _P, _P]),
    "gbf_track": (C.c_int, [_P, _D16, C.POINTER(TrackResult), _P]),
    "gbf_get_image": (C.c_int, [_P, _I32, _I32, _I32, _P, _I64, _P]),
    "gbf_process_frame": (C.c_int, [_P, _P, _I64, _P, _I64, _P]),
    "gbf_process_frame_staged": (C.c_int, [_P, _P]),
    "gbf_map_export": (C.c_int, [_P, _P, _P, _P, _P, _I64, C.POINTER(C.c_int64)]),
    "gbf_map_import": (C.c_int, [_P, _P, _P, _P, _P, _I64]),
    "gbf_raycast_check_visibility": (C.c_int, [_P, _D16, _P, _I64, _P]),
    "gbf_render_scene": (C.c_int, [_P, _I64, _P, _I64, _P, _I64, _I32, _I32, _P, _I64, _P]),
    "gbf_session_render": (C.c_int, [_P, _I32, _P, _I64, _P]),
    "gbf_dump_write": (C.c_int, [C.c_char_p, _P, _P, _P, _P, _P, _I64]),
    "gbf_dump_read": (C.c_int, [C.c_char_p, _P, _P, _P, _P, _P, _I64, C.POINTER(C.c_int64)]),
    "gbf_map_write_dump": (C.c_int, [_P, C.c_char_p, _P]),
    "gbf_map_delete_blocks": (C.c_int, [_P, _P, _I64, C.POINTER(C.c_int64)]),
    "gbf_map_prune": (C.c_int, [_P, _P, C.c_double, _I32, C.POINTER(C.c_int64)]),
    "gbf_map_prune_async": (C.c_int, [_P, _P, C.c_double, _I32, _P]),
    "gbf_session_snapshot_bytes": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "gbf_session_snapshot": (C.c_int, [_P, _P, _I64, C.POINTER(C.c_int64), _P]),
    "gbf_session_restore": (C.c_int, [_P, _P, _I64, _P]),
    "gbf_map_read_dump": (C.c_int, [_P, C.c_char_p]),
    "gbf_visible_blocks": (C.c_int, [_P, _P, _I64, C.POINTER(C.c_int64)]),
    "gbf_zrange": (C.c_int, [_P, _P, _I64]),
    "gbf_batch_create": (C.c_int, [_I32, C.POINTER(_P)]),
    "gbf_batch_destroy": (C.c_int, [_P]),
    "gbf_batch_set": (C.c_int, [_P, _I32, _P]),
    "gbf_batch_reserve": (C.c_int, [_P, C.POINTER(Config), C.POINTER(Intrinsics), _I32]),
    "gbf_batch_process": (C.c_int, [_P, _P, _I32, _P]),
    "gbf_batch_set_inputs": (C.c_int, [_P, _I32, _P, _P]),
    "gbf_batch_set_timing": (C.c_int, [_P, _I32]),
    "gbf_batch_set_groups": (C.c_int, [_P, _I32]),
    "gbf_batch_set_stagger": (C.c_int, [_P, _I32]),
    "gbf_batch_set_ray_tile": (C.c_int, [_P, _I32]),
    "gbf_batch_set_autotune": (C.c_int, [_P, _I32, _I32]),
    "gbf_batch_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "gbf_autotune_forget": (C.c_int, []),
    "gbf_batch_flush": (C.c_int, [_P, _P]),
    "gbf_batch_stage": (C.c_int, [_P, _I32, _P, _I64, _P, _I64, _P]),
    "gbf_batch_results": (C.c_int, [_P, _I32, _P, _I32]),
    "gbf_batch_phase_ms": (C.c_int, [_P, C.POINTER(C.c_float), _I32]),
    "gbf_batch_kernels": (C.c_int, [_P, C.POINTER(_I32)]),
    "gbf_batch_captures": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "gbf_synth_default": (C.c_int, [C.POINTER(SynthParams)]),
    "gbf_synth_create": (C.c_int, [C.POINTER(SynthParams), C.POINTER(_P)]),
    "gbf_synth_destroy": (C.c_int, [_P]),
    "gbf_synth_pose": (C.c_int, [_P, _I32, _D16]),
    "gbf_synth_render": (C.c_int, [_P, C.POINTER(Intrinsics), _D16, _I32, _P, _P, _P]),
}


class GbfError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    """The loaded libgbfusion; raises if it was not built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"libgbfusion is not built ({LIB_PATH} missing); run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != OK:
        msg = lib().gbf_last_error()
        raise GbfError(status, where, msg.decode() if msg else "")


def call(name: str, *args):
    st = getattr(lib(), name)(*args)
    check(st, name)


def mat16(T) -> C.Array:
    """4x4 (or 16) pose -> ctypes double[16], row-major."""
    import numpy as np
    a = np.ascontiguousarray(np.asarray(T, dtype=np.float64).reshape(16))
    return (C.c_double * 16)(*a.tolist())


def default_config(**over) -> Config:
    c = Config()
    call("gbf_config_default", C.byref(c))
    for k, v in over.items():
        if k == "max_iterations":
            for i, x in enumerate(v):
                c.max_iterations[i] = int(x)
        else:
            setattr(c, k, v)
    return c
