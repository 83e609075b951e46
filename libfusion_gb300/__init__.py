"""libfusion_gb300 -- Python mirror of the reference's dense-fusion host API on
top of the libgbfusion C ABI (include/gbfusion.h).

Classes keep the reference's names and method meanings (paths relative to the
reference project):

* ``DenseMapping``  -- include/voxel_hashing/voxel_hashing.h:12-51
* ``DenseTracking`` -- include/tracking/icp_tracker.h:28-88
* ``System``        -- include/system.h:17-95 (``process_images``)

Images are CUDA tensors (torch is only the carrier of device memory): depth
(H, W) float32 metres or uint16 millimetres, colour (H, W, 3) uint8, vertex /
normal maps (H, W, 4) float32.  Poses are 4x4 float64 arrays, camera -> world.
Every call goes to the CUDA kernels; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import (FLAG_COORD_RANGE, FLAG_HASH_FULL, FLAG_NAN_POSE, FLAG_POOL_EXHAUSTED, FLAG_TRACK_FAILED,
                   MESH_COLOUR, MESH_NORMAL, MESH_VERTEX, VOXEL_HALF, VOXEL_REF, VOXEL_SNORM, GbfError, call,
                   default_config, lib, mat16)

__all__ = [
    "IntrinsicMatrix", "DenseMapping", "DenseTracking", "System", "FusionBatch", "SynthScene", "TrackingResult",
    "write_dump", "read_dump", "render_scene", "autotune_forget",
    "default_config", "session_bytes", "GbfError", "VOXEL_REF", "VOXEL_HALF", "VOXEL_SNORM", "MESH_VERTEX", "MESH_NORMAL",
    "MESH_COLOUR", "FLAG_POOL_EXHAUSTED", "FLAG_HASH_FULL", "FLAG_COORD_RANGE", "FLAG_TRACK_FAILED",
    "FLAG_NAN_POSE", "version",
]


def version() -> str:
    return lib().gbf_version().decode()


@dataclass
class IntrinsicMatrix:
    """IntrinsicMatrix (include/data_struct/intrinsic_matrix.h:12-20)."""
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float

    def pyr_down(self) -> "IntrinsicMatrix":
        s = 0.5
        return IntrinsicMatrix(int(s * self.width), int(s * self.height), s * self.fx, s * self.fy, s * self.cx,
                               s * self.cy)

    def c(self) -> _lib.Intrinsics:
        return _lib.Intrinsics(self.width, self.height, self.fx, self.fy, self.cx, self.cy)


@dataclass
class TrackingResult:
    """TrackingResult (include/tracking/icp_tracker.h:13-18) plus diagnostics."""
    sucess: bool
    icp_error: float
    update: np.ndarray
    rgb_error: float = 0.0
    iterations: int = 0
    icp_inliers: float = 0.0
    rgb_inliers: float = 0.0

    @staticmethod
    def of(r: _lib.TrackResult) -> "TrackingResult":
        return TrackingResult(bool(r.success), r.icp_error, np.array(r.update[:], dtype=np.float64).reshape(4, 4),
                              r.rgb_error, r.iterations, r.icp_inliers, r.rgb_inliers)


def session_bytes(cfg: _lib.Config, K: IntrinsicMatrix) -> int:
    """Device bytes of one session (admission control); no GPU needed."""
    out = C.c_uint64()
    kc = K.c()
    call("gbf_session_bytes", C.byref(cfg), C.byref(kc), C.byref(out))
    return int(out.value)


def _ptr(t) -> int:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return t.data_ptr()


def _stream(stream) -> int:
    """cudaStream_t handle of a torch stream, a raw handle, or the current stream (None)."""
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


class _Session:
    """One reconstruction session: map + tracker state resident on the GPU."""

    def __init__(self, K: IntrinsicMatrix, cfg: _lib.Config | None = None):
        self.K = K
        self.cfg = cfg if cfg is not None else default_config()
        self._h = C.c_void_p()
        kc = K.c()
        call("gbf_session_create", C.byref(self.cfg), C.byref(kc), C.byref(self._h))

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            call("gbf_session_destroy", self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def inputs(self):
        """Device staging buffers (u16 depth mm, rgb8) as raw pointers."""
        d, r = C.c_void_p(), C.c_void_p()
        call("gbf_session_inputs", self._h, C.byref(d), C.byref(r))
        return d.value, r.value

    def stage(self, depth_mm, image, stream=None) -> None:
        """Copy a frame (CUDA or pinned CPU tensors) into the staging buffers."""
        W = self.K.width
        call("gbf_session_stage", self._h, depth_mm.data_ptr(), W * 2, image.data_ptr(), W * 3, _stream(stream))

    def stats(self, stream=None) -> _lib.FrameStats:
        s = _lib.FrameStats()
        call("gbf_get_stats", self._h, C.byref(s), _stream(stream))
        return s

    def set_pose(self, T, stream=None) -> None:
        call("gbf_set_pose", self._h, mat16(T), _stream(stream))

    def get_pose(self, stream=None) -> np.ndarray:
        out = (C.c_double * 16)()
        call("gbf_get_pose", self._h, out, _stream(stream))
        return np.array(out[:], dtype=np.float64).reshape(4, 4)

    def reset(self, stream=None) -> None:
        call("gbf_session_reset", self._h, _stream(stream))

    def snapshot_bytes(self) -> int:
        n = C.c_int64()
        call("gbf_session_snapshot_bytes", self._h, C.byref(n))
        return int(n.value)

    def snapshot(self, out=None, stream=None):
        """Everything the session's next frame reads (blocks, tracking state,
        reference pyramid), into `out` (a host numpy uint8 array or a CUDA
        uint8 tensor, large enough) or a new host array; returns it, cut to the
        snapshot's size."""
        n = self.snapshot_bytes()
        if out is None:
            out = np.empty(n, np.uint8)
        ptr = out.ctypes.data if isinstance(out, np.ndarray) else out.data_ptr()
        cap = out.nbytes if isinstance(out, np.ndarray) else out.numel() * out.element_size()
        written = C.c_int64()
        call("gbf_session_snapshot", self._h, ptr, cap, C.byref(written), _stream(stream))
        return out[:int(written.value)]

    def restore(self, snap, stream=None) -> None:
        """Continue from a snapshot of a session of the same configuration and intrinsics."""
        if isinstance(snap, np.ndarray):
            snap = np.ascontiguousarray(snap)
            ptr, n = snap.ctypes.data, snap.nbytes
        else:
            ptr, n = snap.data_ptr(), snap.numel() * snap.element_size()
        call("gbf_session_restore", self._h, ptr, n, _stream(stream))


class DenseMapping(_Session):
    """Voxel-hashed TSDF map (include/voxel_hashing/voxel_hashing.h:12-51)."""

    def update(self, depth, image, pose, normal=None, stream=None) -> None:
        """update(depth, image, pose) -- 1/d^2 colour update; with `normal`
        the normal-weighted update of update(RgbdImagePtr)."""
        W = self.K.width
        call("gbf_fuse", self._h, _ptr(depth), W * 4, _ptr(image), W * 3, _ptr(normal), W * 16, mat16(pose),
             _stream(stream))

    def raycast(self, vmap, pose, nmap=None, rgb=None, stream=None) -> None:
        """Raycast at `pose` into `vmap` (H, W, 4); with `nmap` (H, W, 4) the model
        normals, with `rgb` (H, W, 3) uint8 the hits' voxel colours (white elsewhere)."""
        if nmap is None and rgb is None:
            call("gbf_raycast", self._h, mat16(pose), _ptr(vmap), self.K.width * 16, _stream(stream))
            return
        call("gbf_raycast_maps", self._h, mat16(pose), _ptr(vmap), self.K.width * 16,
             None if nmap is None else _ptr(nmap), self.K.width * 16,
             None if rgb is None else _ptr(rgb), self.K.width * 3, _stream(stream))

    def raycast_check_visibility(self, vmap, pose, stream=None) -> None:
        """Visible blocks recomputed for `pose` (frustum test over every allocated
        block), then raycast at `pose` into `vmap`."""
        call("gbf_raycast_check_visibility", self._h, mat16(pose), _ptr(vmap), self.K.width * 16, _stream(stream))

    def reset_mapping(self, stream=None) -> None:
        self.reset(stream)

    def _mesh(self, mode, vertex, attr, stream=None) -> int:
        n = C.c_uint64()
        max_tris = vertex.numel() // 9
        call("gbf_extract_mesh", self._h, mode, _ptr(vertex), _ptr(attr), max_tris, C.byref(n), _stream(stream))
        return int(n.value)

    def fetch_mesh_vertex_only(self, vertex, stream=None) -> int:
        return self._mesh(MESH_VERTEX, vertex, None, stream)

    def fetch_mesh_with_normal(self, vertex, normal, stream=None) -> int:
        return self._mesh(MESH_NORMAL, vertex, normal, stream)

    def fetch_mesh_with_colour(self, vertex, colour, stream=None) -> int:
        return self._mesh(MESH_COLOUR, vertex, colour, stream)

    def export(self):
        """Allocated blocks in canonical form: coords (n,3) int32, sdf / weight
        (n,512) float32, rgb (n,512,3) uint8."""
        n = C.c_int64()
        call("gbf_map_export", self._h, None, None, None, None, 0, C.byref(n))
        k = int(n.value)
        coords = np.zeros((k, 3), np.int32)
        sdf = np.zeros((k, 512), np.float32)
        w = np.zeros((k, 512), np.float32)
        rgb = np.zeros((k, 512, 3), np.uint8)
        if k:
            call("gbf_map_export", self._h, coords.ctypes.data, sdf.ctypes.data, w.ctypes.data, rgb.ctypes.data, k,
                 C.byref(n))
        return coords, sdf, w, rgb

    def import_blocks(self, coords, sdf, w, rgb) -> None:
        coords = np.ascontiguousarray(coords, np.int32)
        sdf = np.ascontiguousarray(sdf, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        call("gbf_map_import", self._h, coords.ctypes.data, sdf.ctypes.data, w.ctypes.data, rgb.ctypes.data,
             len(coords))

    def writeMapToDisk(self, file_name: str, size: tuple[int, int, int] | None = None) -> None:
        """DenseMapping::writeMapToDisk (src/voxel_hashing/voxel_hashing.cpp:189-196): the
        reference's raw dump (``file_name`` + ``file_name.txt``).  ``size`` =
        (num_blocks, num_hash_entries, num_buckets); None = the reference's
        defaults, which its own reader assumes."""
        ms = None if size is None else C.byref(_lib.MapSize(*size))
        call("gbf_map_write_dump", self._h, str(file_name).encode(), ms)

    def readMapFromDisk(self, file_name: str) -> None:
        """DenseMapping::readMapFromDisk (src/voxel_hashing/voxel_hashing.cpp:198-205):
        replaces the map with the dump's blocks; pose and tracking state stay."""
        call("gbf_map_read_dump", self._h, str(file_name).encode())

    def delete_blocks(self, coords) -> int:
        """Remove the listed blocks (block coordinates); returns how many were removed."""
        c = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        n = C.c_int64()
        call("gbf_map_delete_blocks", self._h, c.ctypes.data if len(c) else None, len(c), C.byref(n))
        return int(n.value)

    def prune(self, center=None, radius: float = -1.0, drop_unobserved: bool = False) -> int:
        """Remove blocks farther than `radius` m from `center` and/or without any
        observed voxel; returns how many were removed."""
        n = C.c_int64()
        ctr = None if center is None else (C.c_double * 3)(*[float(x) for x in center])
        call("gbf_map_prune", self._h, ctr, float(radius), 1 if drop_unobserved else 0, C.byref(n))
        return int(n.value)

    def prune_async(self, center=None, radius: float = -1.0, drop_unobserved: bool = False, stream=None) -> None:
        """prune() enqueued on `stream` (default: torch's current stream) with
        no host synchronisation; stats().allocated_blocks gives what is left."""
        ctr = None if center is None else (C.c_double * 3)(*[float(x) for x in center])
        call("gbf_map_prune_async", self._h, ctr, float(radius), 1 if drop_unobserved else 0, _stream(stream))

    def visible_blocks(self) -> np.ndarray:
        n = C.c_int64()
        call("gbf_visible_blocks", self._h, None, 0, C.byref(n))
        out = np.zeros((int(n.value), 3), np.int32)
        if len(out):
            call("gbf_visible_blocks", self._h, out.ctypes.data, len(out), C.byref(n))
        return out

    def zrange(self) -> np.ndarray:
        cells = (self.K.width // 8) * (self.K.height // 8)
        out = np.zeros((cells, 2), np.float32)
        call("gbf_zrange", self._h, out.ctypes.data, cells)
        return out.reshape(self.K.height // 8, self.K.width // 8, 2)


class DenseTracking(DenseMapping):
    """Pyramid ICP + photometric tracker (include/tracking/icp_tracker.h:28-88)."""

    def set_image(self, which: int, depth, image, stream=None) -> None:
        """Build a frame's pyramids: which=1 reference (`last`), 0 current."""
        W = self.K.width
        call("gbf_build_pyramid", self._h, which, _ptr(depth), W * 4, _ptr(image), W * 3, _stream(stream))

    def set_reference(self, depth, image, stream=None) -> None:
        self.set_image(1, depth, image, stream)

    def set_current(self, depth, image, stream=None) -> None:
        self.set_image(0, depth, image, stream)

    def compute_transform(self, init=None, stream=None) -> TrackingResult:
        r = _lib.TrackResult()
        call("gbf_track", self._h, mat16(np.eye(4) if init is None else init), C.byref(r), _stream(stream))
        return TrackingResult.of(r)

    def reduce(self, level: int, T, stddev: float = 0.0, stream=None) -> np.ndarray:
        out = (C.c_double * 58)()
        call("gbf_reduce", self._h, level, mat16(T), stddev, out, _stream(stream))
        return np.array(out[:], dtype=np.float64)

    def get_image(self, which: int, kind: int, level: int, stream=None):
        import torch
        K = self.K
        for _ in range(level):
            K = K.pyr_down()
        ch = 4 if kind in (0, 1) else 1
        t = torch.empty((K.height, K.width, ch) if ch == 4 else (K.height, K.width), dtype=torch.float32,
                        device="cuda")
        call("gbf_get_image", self._h, which, kind, level, t.data_ptr(), K.width * 4 * ch, _stream(stream))
        return t


class System(DenseTracking):
    """Per-frame fusion loop (System::process_images, src/system.cpp:40-114)."""

    def process_images(self, depth_mm, image, stream=None) -> None:
        W = self.K.width
        call("gbf_process_frame", self._h, _ptr(depth_mm), W * 2, _ptr(image), W * 3, _stream(stream))

    def process_staged(self, stream=None) -> None:
        call("gbf_process_frame_staged", self._h, _stream(stream))

    def get_camera_pose(self, stream=None) -> np.ndarray:
        return self.get_pose(stream)

    def _render(self, textured: bool, stream=None):
        import torch
        out = torch.empty((self.K.height, self.K.width, 4), dtype=torch.uint8, device="cuda")
        call("gbf_session_render", self._h, 1 if textured else 0, out.data_ptr(), self.K.width * 4, _stream(stream))
        return out

    def get_rendered_image(self, stream=None):
        """Phong-shaded model prediction, (H, W, 4) uint8 on the device."""
        return self._render(False, stream)

    def get_rendered_scene_textured(self, stream=None):
        """The same shading with the last frame's colour."""
        return self._render(True, stream)


class FusionBatch:
    """Many sessions processed in the same launches (one frame each per tick)."""

    def __init__(self, max_sessions: int):
        self._h = C.c_void_p()
        self.max = max_sessions
        self.slots: list[System | None] = [None] * max_sessions
        call("gbf_batch_create", max_sessions, C.byref(self._h))

    def set(self, slot: int, session: System | None) -> None:
        call("gbf_batch_set", self._h, slot, session.handle if session is not None else None)
        self.slots[slot] = session

    def reserve(self, K: IntrinsicMatrix, cfg: _lib.Config, slots: int) -> None:
        """Size the tick for `slots` sessions no larger than (K, cfg), so that
        sessions of up to that size come and go without a new captured graph."""
        kc = K.c()
        call("gbf_batch_reserve", self._h, C.byref(cfg), C.byref(kc), slots)

    def set_inputs(self, slot: int, depth_ptr: int | None, rgb_ptr: int | None) -> None:
        """Take slot's next frame from these device pointers (dense u16, rgb8)."""
        call("gbf_batch_set_inputs", self._h, slot, depth_ptr, rgb_ptr)

    def process(self, active, use_graph: bool = True, stream=None) -> None:
        a = (C.c_uint8 * self.max)(*[1 if x else 0 for x in active])
        call("gbf_batch_process", self._h, a, 1 if use_graph else 0, _stream(stream))

    PHASES = ("ingest", "track", "alloc_visible", "integrate", "zrange", "march", "post")

    def set_timing(self, enable: bool) -> None:
        call("gbf_batch_set_timing", self._h, 1 if enable else 0)

    def stage(self, slot: int, depth, rgb, stream=None) -> None:
        """Copy slot's frame for the next tick (host or device tensors: depth
        (H, W) uint16 mm, rgb (H, W, 3) uint8) into the batch's double-buffered
        inputs on `stream`; ordered on the device against the ticks."""
        W = depth.shape[-1]
        call("gbf_batch_stage", self._h, int(slot), depth.data_ptr(), W * 2, rgb.data_ptr(), W * 3, _stream(stream))

    def results(self, back: int = 0):
        """Outcome of the last submitted tick (back=0) or the one before (back=1):
        poses (n, 4, 4) camera->world, tracked (n,), status (n,), frame_index (n,)."""
        arr = (_lib.SlotResult * self.max)()
        call("gbf_batch_results", self._h, int(back), arr, self.max)
        poses = np.array([list(x.pose) for x in arr]).reshape(self.max, 4, 4)
        return (poses, np.array([x.tracked for x in arr], np.int32), np.array([x.status for x in arr], np.uint32),
                np.array([x.frame_index for x in arr], np.int64))

    def set_stagger(self, enable: bool) -> None:
        """Odd session groups half a frame out of phase (same results)."""
        call("gbf_batch_set_stagger", self._h, 1 if enable else 0)

    def set_ray_tile(self, tile_w: int) -> None:
        """Raycast tile of the ticks: 64 pixels, tile_w (4, 8, 16, 32) wide (same results)."""
        call("gbf_batch_set_ray_tile", self._h, int(tile_w))

    def autotune(self, enable: bool = True, ticks_per_candidate: int = 6) -> None:
        """Online tuning of groups, stagger and raycast tile while the batch serves
        (gbf_batch_set_autotune); the choice is kept per batch shape for the process."""
        call("gbf_batch_set_autotune", self._h, 1 if enable else 0, int(ticks_per_candidate))

    def tuning(self) -> dict:
        """The tuner's state: 'off' / 'exploring' / 'settled', the shape in use and
        the median tick time of every candidate timed."""
        t = _lib.Tuning()
        call("gbf_batch_tuning", self._h, C.byref(t))
        shape = lambda s: {"groups": s.groups, "stagger": s.stagger, "ray_tile_w": s.ray_tile_w,
                           "median_ms": s.median_ms}
        return {"state": ("off", "exploring", "settled")[t.state], "from_table": bool(t.from_table),
                "ticks_per_candidate": t.ticks_per_candidate, "chosen": shape(t.chosen),
                "tried": [shape(t.tried[i]) for i in range(t.n_tried)]}

    def flush(self, stream=None) -> None:
        """Fuse what the staggered groups owe; call before reading a batched session's map."""
        call("gbf_batch_flush", self._h, _stream(stream))

    def set_groups(self, groups: int) -> None:
        """Run the slots as `groups` concurrent branches of each tick (1..4)."""
        call("gbf_batch_set_groups", self._h, int(groups))

    def phase_ms(self) -> dict:
        """Mean per-phase milliseconds over the ticks since set_timing(True)."""
        out = (C.c_float * 8)()
        call("gbf_batch_phase_ms", self._h, out, 8)
        d = dict(zip(self.PHASES, out[:7]))
        d["ticks"] = int(out[7])
        return d

    def captures(self) -> int:
        """Tick graphs captured so far."""
        n = C.c_int64()
        call("gbf_batch_captures", self._h, C.byref(n))
        return int(n.value)

    def kernels_per_tick(self) -> int:
        n = C.c_int32()
        call("gbf_batch_kernels", self._h, C.byref(n))
        return int(n.value)

    def close(self) -> None:
        """Destroy the batch and let go of the sessions in its slots (they stay
        usable on their own)."""
        if self._h:
            call("gbf_batch_destroy", self._h)
            self._h = C.c_void_p()
        self.slots = [None] * len(self.slots)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_forget() -> None:
    """Clear the process-wide table of tuned batch shapes (gbf_autotune_forget)."""
    call("gbf_autotune_forget")


def render_scene(vmap, nmap, rgb=None, stream=None):
    """renderScene / renderSceneTextured: (H, W, 4) float32 camera-frame vertex and
    normal maps (CUDA tensors), optional (H, W, 3) uint8 colour -> (H, W, 4) uint8."""
    import torch
    h, w = vmap.shape[:2]
    out = torch.empty((h, w, 4), dtype=torch.uint8, device=vmap.device)
    call("gbf_render_scene", _ptr(vmap), w * 16, _ptr(nmap), w * 16, None if rgb is None else _ptr(rgb), w * 3,
         w, h, out.data_ptr(), w * 4, _stream(stream))
    return out


def write_dump(file_name: str, coords, sdf, weight, rgb, size: tuple[int, int, int] | None = None) -> None:
    """Reference raw map dump from canonical per-block arrays (host only, no device)."""
    coords = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
    n = len(coords)
    sdf = np.ascontiguousarray(sdf, np.float32).reshape(n, 512)
    weight = np.ascontiguousarray(weight, np.float32).reshape(n, 512)
    rgb = np.ascontiguousarray(rgb, np.uint8).reshape(n, 512, 3)
    ms = None if size is None else C.byref(_lib.MapSize(*size))
    call("gbf_dump_write", str(file_name).encode(), ms, coords.ctypes.data, sdf.ctypes.data, weight.ctypes.data,
         rgb.ctypes.data, n)


def read_dump(file_name: str):
    """Blocks of a reference raw map dump (host only): (coords, sdf, weight, rgb, size)."""
    ms = _lib.MapSize()
    n = C.c_int64()
    call("gbf_dump_read", str(file_name).encode(), C.byref(ms), None, None, None, None, 0, C.byref(n))
    k = int(n.value)
    coords = np.zeros((k, 3), np.int32)
    sdf = np.zeros((k, 512), np.float32)
    w = np.zeros((k, 512), np.float32)
    rgb = np.zeros((k, 512, 3), np.uint8)
    if k:
        call("gbf_dump_read", str(file_name).encode(), None, coords.ctypes.data, sdf.ctypes.data, w.ctypes.data,
             rgb.ctypes.data, k, C.byref(n))
    return coords, sdf, w, rgb, (ms.num_blocks, ms.num_hash_entries, ms.num_buckets)


class SynthScene:
    """Seeded synthetic room (spheres + boxes) rendered to u16 depth + rgb8."""

    def __init__(self, **over):
        p = _lib.SynthParams()
        call("gbf_synth_default", C.byref(p))
        for k, v in over.items():
            if k == "room":
                for i, x in enumerate(v):
                    p.room[i] = float(x)
            else:
                setattr(p, k, v)
        self.params = p
        self._h = C.c_void_p()
        call("gbf_synth_create", C.byref(p), C.byref(self._h))

    def pose(self, frame: int) -> np.ndarray:
        out = (C.c_double * 16)()
        call("gbf_synth_pose", self._h, frame, out)
        return np.array(out[:], dtype=np.float64).reshape(4, 4)

    def render(self, K: IntrinsicMatrix, frame: int, pose=None, depth=None, rgb=None, stream=None):
        import torch
        T = self.pose(frame) if pose is None else pose
        if depth is None:
            depth = torch.empty((K.height, K.width), dtype=torch.uint16, device="cuda")
        if rgb is None:
            rgb = torch.empty((K.height, K.width, 3), dtype=torch.uint8, device="cuda")
        kc = K.c()
        call("gbf_synth_render", self._h, C.byref(kc), mat16(T), frame, depth.data_ptr(), rgb.data_ptr(),
             _stream(stream))
        return depth, rgb

    def render_into(self, K: IntrinsicMatrix, frame: int, depth_ptr: int, rgb_ptr: int, pose=None, stream=None):
        T = self.pose(frame) if pose is None else pose
        kc = K.c()
        call("gbf_synth_render", self._h, C.byref(kc), mat16(T), frame, depth_ptr, rgb_ptr, _stream(stream))

    def close(self):
        if self._h:
            call("gbf_synth_destroy", self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
