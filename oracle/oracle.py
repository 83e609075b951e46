"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker, never as the product.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
MAX_LEVELS = 5


class OrConfig(C.Structure):
    _fields_ = [
        ("voxel_size", C.c_float), ("truncation", C.c_float),
        ("zmin_update", C.c_float), ("zmax_update", C.c_float),
        ("zmin_raycast", C.c_float), ("zmax_raycast", C.c_float),
        ("num_blocks", C.c_int32), ("voxel_layout", C.c_int32), ("num_levels", C.c_int32),
        ("max_iterations", C.c_int32 * MAX_LEVELS),
        ("w_icp", C.c_float), ("w_rgb", C.c_float), ("icp_dist_thresh", C.c_float),
        ("icp_angle_thresh", C.c_float), ("bilateral", C.c_int32), ("motion_prior", C.c_int32),
        ("threads", C.c_int32),
    ]


class OrIntrinsics(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float)]


class OrTrackResult(C.Structure):
    _fields_ = [("success", C.c_int32), ("iterations", C.c_int32), ("icp_error", C.c_float),
                ("rgb_error", C.c_float), ("icp_inliers", C.c_float), ("rgb_inliers", C.c_float),
                ("update", C.c_double * 16)]


def build() -> Path:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        P, D = C.c_void_p, C.POINTER(C.c_double)
        for s in ("f32", "f64"):
            sig = {
                f"or_map_create_{s}": (P, [C.POINTER(OrConfig), C.POINTER(OrIntrinsics)]),
                f"or_map_destroy_{s}": (None, [P]),
                f"or_fuse_{s}": (C.c_int, [P, P, P, P, D]),
                f"or_raycast_{s}": (C.c_int, [P, D, P]),
                f"or_raycast_check_visibility_{s}": (C.c_int, [P, D, P]),
                f"or_map_blocks_{s}": (C.c_int64, [P]),
                f"or_ray_stats_{s}": (None, [P, D, C.POINTER(C.c_longlong), P]),
                f"or_map_export_{s}": (C.c_int64, [P, P, P, P, P, C.c_int64]),
                f"or_visible_{s}": (C.c_int64, [P, P, C.c_int64]),
                f"or_zrange_{s}": (None, [P, P]),
                f"or_render_blocks_{s}": (C.c_int32, [P]),
                f"or_mesh_{s}": (C.c_int64, [P, C.c_int, P, P, C.c_int64]),
                f"or_frame_create_{s}": (P, [C.POINTER(OrConfig), C.POINTER(OrIntrinsics)]),
                f"or_frame_destroy_{s}": (None, [P]),
                f"or_build_pyramid_{s}": (None, [P, P, P]),
                f"or_frame_get_{s}": (None, [P, C.c_int, C.c_int, P]),
                f"or_frame_set_vmap_{s}": (None, [P, P]),
                f"or_reduce_{s}": (None, [P, P, C.c_int, C.POINTER(C.c_float), C.c_float, D]),
                f"or_reduce_terms_{s}": (None, [P, P, C.c_int, C.POINTER(C.c_float), C.c_float, P]),
                f"or_raycast_maps_{s}": (C.c_int, [P, D, P, P]),
                f"or_track_{s}": (None, [P, P, D, C.POINTER(OrTrackResult)]),
                f"or_system_create_{s}": (P, [C.POINTER(OrConfig), C.POINTER(OrIntrinsics)]),
                f"or_system_destroy_{s}": (None, [P]),
                f"or_system_set_pose_{s}": (None, [P, D]),
                f"or_system_get_pose_{s}": (None, [P, D]),
                f"or_process_frame_{s}": (None, [P, P, P]),
                f"or_system_map_{s}": (P, [P]),
                f"or_system_ref_{s}": (P, [P]),
                f"or_system_last_result_{s}": (None, [P, C.POINTER(OrTrackResult)]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
        L.or_compute_hash.restype = C.c_int
        L.or_compute_hash.argtypes = [C.c_int] * 4
        L.or_floor_ref.restype = C.c_int
        L.or_floor_ref.argtypes = [C.c_float]
        L.or_voxel_to_block.argtypes = [P, P]
        L.or_voxel_to_local.argtypes = [P, P]
        L.or_local_idx.restype = C.c_int
        L.or_local_idx.argtypes = [P]
        L.or_tri_table.restype = C.c_int
        L.or_tri_table.argtypes = [C.c_int, P]
        L.or_edge_table.restype = C.c_int
        L.or_edge_table.argtypes = [C.c_int]
        L.or_pack_sdf.restype = C.c_short
        L.or_pack_sdf.argtypes = [C.c_float]
        L.or_unpack_sdf.restype = C.c_float
        L.or_unpack_sdf.argtypes = [C.c_short]
        L.or_render_scene.restype = None
        L.or_render_scene.argtypes = [P, P, P, C.c_int, C.c_int, P]
        L.or_sum_f32.restype = None
        L.or_sum_f32.argtypes = [P, C.c_longlong, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.or_trans_record.restype = None
        L.or_trans_record.argtypes = [C.c_int]
        L.or_trans_recorded.restype = C.c_longlong
        L.or_trans_recorded.argtypes = [C.c_int, P, C.c_longlong]
        L.or_trans_table.restype = None
        L.or_trans_table.argtypes = [C.c_int, P, P, C.c_longlong]
        L.or_trans_misses.restype = C.c_longlong
        L.or_trans_misses.argtypes = [C.c_int]
        _lib = L
    return _lib


def config_from(gcfg, threads: int = 0) -> OrConfig:
    """Oracle config from a libgbfusion Config (same field meanings)."""
    c = OrConfig()
    for f, _ in OrConfig._fields_:
        if f == "threads":
            continue
        if f == "max_iterations":
            for i in range(MAX_LEVELS):
                c.max_iterations[i] = gcfg.max_iterations[i]
        else:
            setattr(c, f, getattr(gcfg, f))
    c.threads = threads
    return c


def intrinsics_from(K) -> OrIntrinsics:
    return OrIntrinsics(K.width, K.height, K.fx, K.fy, K.cx, K.cy)


def _d16(T):
    a = np.ascontiguousarray(np.asarray(T, np.float64).reshape(16))
    return (C.c_double * 16)(*a.tolist())


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


class OracleMap:
    def __init__(self, cfg: OrConfig, K: OrIntrinsics, precision: str = "f32"):
        self.s = precision
        self.cfg, self.K = cfg, K
        self.h = getattr(lib(), f"or_map_create_{precision}")(C.byref(cfg), C.byref(K))

    def fn(self, name):
        return getattr(lib(), f"{name}_{self.s}")

    def fuse(self, depth: np.ndarray, rgb: np.ndarray, pose, nmap: np.ndarray | None = None) -> int:
        depth = np.ascontiguousarray(depth, np.float32)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        nmap = None if nmap is None else np.ascontiguousarray(nmap, np.float32)
        return self.fn("or_fuse")(self.h, _p(depth), _p(rgb), _p(nmap), _d16(pose))

    def raycast(self, pose, vmap: np.ndarray | None = None) -> np.ndarray:
        if vmap is None:
            vmap = np.full((self.K.height, self.K.width, 4), np.nan, np.float32)
        self.fn("or_raycast")(self.h, _d16(pose), _p(vmap))
        return vmap

    def raycast_maps(self, pose):
        """Vertex map and the hits' nearest voxel colours (white elsewhere)."""
        vmap = np.full((self.K.height, self.K.width, 4), np.nan, np.float32)
        rgb = np.full((self.K.height, self.K.width, 3), 255, np.uint8)
        self.fn("or_raycast_maps")(self.h, _d16(pose), _p(vmap), _p(rgb))
        return vmap, rgb

    def raycast_check_visibility(self, pose, vmap: np.ndarray | None = None) -> np.ndarray:
        """DenseMapping::raycast_check_visibility: visible list for `pose`, then raycast."""
        if vmap is None:
            vmap = np.full((self.K.height, self.K.width, 4), np.nan, np.float32)
        self.fn("or_raycast_check_visibility")(self.h, _d16(pose), _p(vmap))
        return vmap

    def ray_stats(self, pose, per_pixel: bool = False):
        """March counts of a raycast at `pose` (rays, steps, voxel samples,
        trilinear reads, hits, steps through unallocated or unobserved space,
        nearest reads in unallocated blocks);
        with per_pixel, also each pixel's cost in samples (steps + 8 per
        trilinear read)."""
        out = (C.c_longlong * 7)()
        pp = np.zeros((self.K.height, self.K.width), np.int32) if per_pixel else None
        self.fn("or_ray_stats")(self.h, _d16(pose), out, _p(pp))
        d = dict(zip(("rays", "steps", "samples", "interps", "hits", "empty", "missing"), out[:]))
        return (d, pp) if per_pixel else d

    def export(self):
        n = self.fn("or_map_blocks")(self.h)
        coords = np.zeros((n, 3), np.int32)
        sdf = np.zeros((n, 512), np.float32)
        w = np.zeros((n, 512), np.float32)
        rgb = np.zeros((n, 512, 3), np.uint8)
        self.fn("or_map_export")(self.h, _p(coords), _p(sdf), _p(w), _p(rgb), n)
        return coords, sdf, w, rgb

    def visible(self) -> np.ndarray:
        n = self.fn("or_visible")(self.h, None, 0)
        out = np.zeros((n, 3), np.int32)
        self.fn("or_visible")(self.h, _p(out), n)
        return out

    def zrange(self) -> np.ndarray:
        out = np.zeros((self.K.height // 8, self.K.width // 8, 2), np.float32)
        self.fn("or_zrange")(self.h, _p(out))
        return out

    def render_blocks(self) -> int:
        return self.fn("or_render_blocks")(self.h)

    def mesh(self, mode: int, max_tris: int = 1 << 22):
        vtx = np.zeros((max_tris, 3, 3), np.float32)
        attr = None
        if mode == 1:
            attr = np.zeros((max_tris, 3, 3), np.float32)
        elif mode == 2:
            attr = np.zeros((max_tris, 3, 3), np.uint8)
        n = self.fn("or_mesh")(self.h, mode, _p(vtx), _p(attr), max_tris)
        n = min(n, max_tris)
        return vtx[:n], (attr[:n] if attr is not None else None)

    def __del__(self):
        try:
            self.fn("or_map_destroy")(self.h)
        except Exception:
            pass


class OracleFrame:
    def __init__(self, cfg: OrConfig, K: OrIntrinsics, precision: str = "f32", handle=None, owner=None):
        self.s, self.cfg, self.K = precision, cfg, K
        self._own = handle is None
        self._owner = owner
        self.h = getattr(lib(), f"or_frame_create_{precision}")(C.byref(cfg), C.byref(K)) if handle is None else handle

    def fn(self, name):
        return getattr(lib(), f"{name}_{self.s}")

    def build(self, depth_m: np.ndarray, rgb: np.ndarray) -> None:
        depth_m = np.ascontiguousarray(depth_m, np.float32)
        rgb = np.ascontiguousarray(rgb, np.uint8)
        self.fn("or_build_pyramid")(self.h, _p(depth_m), _p(rgb))

    def get(self, kind: int, level: int) -> np.ndarray:
        w, h = self.K.width >> level, self.K.height >> level
        out = np.zeros((h, w, 4) if kind in (0, 1) else (h, w), np.float32)
        self.fn("or_frame_get")(self.h, kind, level, _p(out))
        return out

    def set_vmap(self, vmap0: np.ndarray) -> None:
        self.fn("or_frame_set_vmap")(self.h, _p(np.ascontiguousarray(vmap0, np.float32)))

    def __del__(self):
        if self._own:
            try:
                self.fn("or_frame_destroy")(self.h)
            except Exception:
                pass


def reduce(ref: OracleFrame, cur: OracleFrame, level: int, T, stddev: float = 0.0) -> np.ndarray:
    Tf = (C.c_float * 12)(*np.asarray(T, np.float64).reshape(-1)[:12].astype(np.float32).tolist())
    out = (C.c_double * 58)()
    getattr(lib(), f"or_reduce_{ref.s}")(ref.h, cur.h, level, Tf, stddev, out)
    return np.array(out[:])


def reduce_terms(ref: OracleFrame, cur: OracleFrame, level: int, T, stddev: float = 0.0) -> np.ndarray:
    """The float terms reduce() adds, per pixel: (pixels, 58)."""
    Tf = (C.c_float * 12)(*np.asarray(T, np.float64).reshape(-1)[:12].astype(np.float32).tolist())
    K = ref.K
    w, h = K.width >> level, K.height >> level
    out = np.zeros((w * h, 58), np.float32)
    getattr(lib(), f"or_reduce_terms_{ref.s}")(ref.h, cur.h, level, Tf, stddev, _p(out))
    return out


def sum_f32(terms: np.ndarray, kahan: bool) -> np.ndarray:
    """Sequential float column sums of terms, plain or Kahan-compensated."""
    t = np.ascontiguousarray(terms, np.float32)
    out = (C.c_double * t.shape[1])()
    lib().or_sum_f32(_p(t), t.shape[0], t.shape[1], 1 if kahan else 0, out)
    return np.array(out[:])


def track(ref: OracleFrame, cur: OracleFrame, init=None):
    r = OrTrackResult()
    getattr(lib(), f"or_track_{ref.s}")(ref.h, cur.h, _d16(np.eye(4) if init is None else init), C.byref(r))
    return r


class OracleSystem:
    def __init__(self, cfg: OrConfig, K: OrIntrinsics, precision: str = "f32"):
        self.s, self.cfg, self.K = precision, cfg, K
        self.h = getattr(lib(), f"or_system_create_{precision}")(C.byref(cfg), C.byref(K))

    def fn(self, name):
        return getattr(lib(), f"{name}_{self.s}")

    def set_pose(self, T) -> None:
        self.fn("or_system_set_pose")(self.h, _d16(T))

    def pose(self) -> np.ndarray:
        out = (C.c_double * 16)()
        self.fn("or_system_get_pose")(self.h, out)
        return np.array(out[:]).reshape(4, 4)

    def process(self, depth_mm: np.ndarray, rgb: np.ndarray) -> None:
        self.fn("or_process_frame")(self.h, _p(np.ascontiguousarray(depth_mm, np.uint16)),
                                    _p(np.ascontiguousarray(rgb, np.uint8)))

    def last_result(self) -> OrTrackResult:
        r = OrTrackResult()
        self.fn("or_system_last_result")(self.h, C.byref(r))
        return r

    def map_export(self):
        m = OracleMap.__new__(OracleMap)
        m.s, m.cfg, m.K = self.s, self.cfg, self.K
        m.h = self.fn("or_system_map")(self.h)
        out = m.export()
        m.h = None
        return out

    def ref_frame(self) -> OracleFrame:
        return OracleFrame(self.cfg, self.K, self.s, handle=self.fn("or_system_ref")(self.h), owner=self)

    def __del__(self):
        try:
            self.fn("or_system_destroy")(self.h)
        except Exception:
            pass


# ---- reference raw map dump (MapStruct::writeToDisk, src/data_struct/map_struct.cu:535-573) ----

REF_VOXEL = np.dtype([("sdf", "<i2"), ("pad0", "<i2"), ("weight", "<f4"), ("rgb", "u1", 3), ("pad1", "u1")])
REF_ENTRY = np.dtype([("ptr", "<i4"), ("offset", "<i4"), ("pos", "<i4", 3)])
REF_DEFAULT_SIZE = (200000, 250000, 200000)  # MapStruct() defaults, map_struct.cu:19-21


TRANS_SIN, TRANS_EXP, TRANS_POW20 = 0, 1, 2


def trans_record(enable: bool) -> None:
    """Start (clearing) or stop recording the FP32 oracle's sinf / expf arguments."""
    lib().or_trans_record(1 if enable else 0)


def trans_recorded(kind: int) -> np.ndarray:
    """The recorded arguments of one kind, unique, as float32."""
    L = lib()
    n = L.or_trans_recorded(kind, None, 0)
    out = np.empty(n, np.uint32)
    if n:
        L.or_trans_recorded(kind, out.ctypes.data, n)
    return np.unique(out).view(np.float32)


def trans_table(kind: int, x: np.ndarray | None = None, y: np.ndarray | None = None) -> None:
    """Install the values y = f(x) for the FP32 oracle's sinf (kind 0) or expf
    (kind 1); None removes the table.  x: unique float32 arguments."""
    L = lib()
    if x is None:
        L.or_trans_table(kind, None, None, 0)
        return
    xb = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32)
    order = np.argsort(xb, kind="stable")
    xs = np.ascontiguousarray(xb[order])
    ys = np.ascontiguousarray(np.asarray(y, np.float32)[order])
    L.or_trans_table(kind, xs.ctypes.data, ys.ctypes.data, len(xs))


def trans_misses(kind: int) -> int:
    return int(lib().or_trans_misses(kind))


def with_device_transcendentals(run, device_fns):
    """run() twice: once recording the FP32 oracle's transcendental arguments,
    then with device_fns[kind](x) -> y (the device's sinf / expf of those
    arguments) installed as tables.  Returns the second run's result and the
    table sizes; the tables are removed afterwards.  The oracle's own
    arithmetic is unchanged: only the two functions' values come from the device."""
    trans_record(True)
    try:
        run()
    finally:
        trans_record(False)
    sizes = {}
    for kind, fn in device_fns.items():
        x = trans_recorded(kind)
        sizes[kind] = len(x)
        trans_table(kind, x, fn(x) if len(x) else x)
    try:
        out = run()
        misses = {k: trans_misses(k) for k in device_fns}
    finally:
        for kind in device_fns:
            trans_table(kind, None)
    return out, sizes, misses


def parse_ref_dump(path) -> dict:
    """The arrays of a raw dump, in writeToDisk's order: voxels (Voxel, voxel.h:20-22),
    hash table (HashEntry, hash_entry.h:20-22), heap, bucket mutexes, heap counter,
    excess counter; sizes from "<path>.txt" (MapSize, map_struct.h:53-58)."""
    path = Path(path)
    txt = Path(str(path) + ".txt")
    nb, ne, nbk = (np.fromfile(txt, "<i4", 3).tolist() if txt.exists() else REF_DEFAULT_SIZE)
    raw = np.fromfile(path, np.uint8)
    out, off = {"size": (nb, ne, nbk)}, 0
    for name, dt, cnt in (("voxels", REF_VOXEL, nb * 512), ("table", REF_ENTRY, ne), ("heap", np.dtype("<i4"), nb),
                          ("mutex", np.dtype("<i4"), nbk), ("heap_counter", np.dtype("<i4"), 1),
                          ("excess_counter", np.dtype("<i4"), 1)):
        nbytes = dt.itemsize * cnt
        out[name] = raw[off:off + nbytes].view(dt)
        off += nbytes
    if off != raw.size:
        raise ValueError(f"dump is {raw.size} bytes, its MapSize implies {off}")
    return out


def ref_compute_hash(x: int, y: int, z: int, n: int) -> int:
    """computeHash (map_struct.cu:143-148): int32 wraparound products, C remainder, made non-negative."""
    def i32(v):
        return ((v + 2**31) % 2**32) - 2**31
    h = i32(i32(x * 73856093) ^ i32(y * 19349669) ^ i32(z * 83492791))
    r = abs(h) % n * (1 if h >= 0 else -1)  # C remainder takes the dividend's sign
    return r + n if r < 0 else r


def ref_find_entry(dump: dict, pos) -> int:
    """findEntry (map_struct.cu:365-380): index of the live entry for block `pos`
    along its bucket's excess chain, or -1."""
    table, nbk = dump["table"], dump["size"][2]
    i = ref_compute_hash(int(pos[0]), int(pos[1]), int(pos[2]), nbk)
    while True:
        e = table[i]
        if e["ptr"] != -1 and tuple(e["pos"]) == tuple(int(p) for p in pos):
            return i
        if e["offset"] <= 0:
            return -1
        i = nbk + int(e["offset"]) - 1


def render_scene(vmap: np.ndarray, nmap: np.ndarray, rgb: np.ndarray | None = None) -> np.ndarray:
    """renderScene / renderSceneTextured (cuda_imgproc.cu:17-108): (H, W, 4) float32
    camera-frame vertex and normal maps, optional (H, W, 3) uint8 colour -> (H, W, 4) uint8."""
    h, w = vmap.shape[:2]
    vmap = np.ascontiguousarray(vmap, np.float32)
    nmap = np.ascontiguousarray(nmap, np.float32)
    out = np.zeros((h, w, 4), np.uint8)
    c = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
    lib().or_render_scene(_p(vmap), _p(nmap), _p(c), w, h, _p(out))
    return out
