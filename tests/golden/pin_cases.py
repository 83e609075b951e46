"""The cases of the reference-kernel pins (tests/golden/ref_kernels.npz) and
the oracle's side of each.

The reference's integration, z-range / raycast, ICP-row and photometric-row
kernels (src/voxel_hashing/depth_fusion.cu:288-428, ray_tracing.cu:17-425,
src/tracking/pose_estimator.cu:166-222, m_estimator.cu:313-391) were compiled
from its own sources (oracle/ref_pin/build_kernels.sh) and run on a GB300 by
tests/golden/make_kernel_golden.py on the inputs defined here; the fixture
holds their outputs.  tests/test_ref_kernel_pins.py recomputes each case with
the oracle and compares.

Inputs: two synthetic RGB-D frames (the seed-0 room, frames 0 and 4) at
96x72, stored in the fixture, and the reference's own map settings: voxel
2 cm, truncation 5 x voxel (MapState::truncation_dist, map_struct.cu:120-123),
update and raycast range 0.3-4 m.  Every derived input (metric depth, normal
maps, vertex maps, intensities, gradients, visible-block lists) is computed
by the oracle from the stored frames with arithmetic only (no bilateral
filter, whose exp would differ between libm builds), so both machines derive
the same bits; the fixture carries digests of the derived images to show it.
"""
from __future__ import annotations

import hashlib

import numpy as np

W, H = 96, 72
FX = FY = 78.75
CX, CY = 47.5, 35.5
FRAMES = (0, 4)          # seed-0 room: reference (A) and current (B) frame
VOXEL = np.float32(0.02)
TAU = np.float32(np.float32(5.0) * VOXEL)  # 5.0f * voxel_size, as the reference computes it
ZMIN, ZMAX = 0.3, 4.0
STDDEVS = (0.0, 8.0)     # photometric sigma: Huber off (iteration 0) and on
LEVELS = (0, 1)
N_SUBSET = 32            # blocks whose voxels the fixture stores in full
N_SAMPLE = 512           # pixels whose rows the fixture stores in full, per case


def intrinsics(L):
    return L.IntrinsicMatrix(W, H, FX, FY, CX, CY)


def config(L):
    return L.default_config(voxel_size=float(VOXEL), truncation=float(TAU), zmin_update=ZMIN, zmax_update=ZMAX,
                            zmin_raycast=ZMIN, zmax_raycast=ZMAX, num_buckets=1 << 15, num_blocks=1 << 13,
                            voxel_layout=0, num_levels=3, bilateral=0, max_probe=1 << 15)


def depth_m(d_u16):
    return d_u16.astype(np.float32) * np.float32(0.001)


def pose_inv(T) -> np.ndarray:
    """The oracle's SE(3) inverse (oracle_impl.h pose_inv), same operation
    order, as 12 row-major doubles; Python floats round every operation."""
    p = [float(x) for x in np.asarray(T, np.float64).reshape(-1)[:12]]
    o = [0.0] * 12
    o[0], o[1], o[2] = p[0], p[4], p[8]
    o[4], o[5], o[6] = p[1], p[5], p[9]
    o[8], o[9], o[10] = p[2], p[6], p[10]
    o[3] = -((o[0] * p[3] + o[1] * p[7]) + o[2] * p[11])
    o[7] = -((o[4] * p[3] + o[5] * p[7]) + o[6] * p[11])
    o[11] = -((o[8] * p[3] + o[9] * p[7]) + o[10] * p[11])
    return np.array(o, np.float64)


def f12(m) -> np.ndarray:
    """A pose as the kernels take it: 12 row-major floats (Sophus cast<float>)."""
    return np.asarray(m, np.float64).reshape(-1)[:12].astype(np.float32)


def relative(T_ref, T_cur) -> np.ndarray:
    """Reference -> current transform of two camera->world poses."""
    return np.linalg.inv(np.asarray(T_cur, np.float64)) @ np.asarray(T_ref, np.float64)


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(f"{a.dtype.str}{a.shape}".encode())
        h.update(a.tobytes())
    return h.hexdigest()


def canonical_nan(a: np.ndarray) -> np.ndarray:
    """NaNs as one bit pattern (the reference writes 0x7fffffff, the oracle the
    default quiet NaN); every other value keeps its bits."""
    a = np.array(a, copy=True)
    a[np.isnan(a)] = np.nan
    return a


# ---------------------------------------------------------------- map states

def map_state_from_oracle(coords, sdf, w, rgb):
    """Canonical map state (blocks sorted by coordinate): coords, int16 sdf
    codes, float weights, rgb.  The oracle's REF voxels hold code / 32767.f,
    from which the code is recovered exactly."""
    code = np.rint(sdf.astype(np.float64) * 32767.0).astype(np.int16)
    assert np.array_equal(code.astype(np.float32) / np.float32(32767), sdf), "not a REF-layout map"
    return canonical_state(coords, code, w, rgb)


def canonical_state(coords, code, w, rgb):
    coords = np.asarray(coords, np.int32).reshape(-1, 3)
    order = np.lexsort((coords[:, 2], coords[:, 1], coords[:, 0]))
    return (coords[order], np.asarray(code, np.int16).reshape(-1, 512)[order],
            np.asarray(w, np.float32).reshape(-1, 512)[order], np.asarray(rgb, np.uint8).reshape(-1, 512, 3)[order])


def subset_rows(coords, chosen) -> np.ndarray:
    """Indices of the chosen block coordinates in a canonical state."""
    index = {tuple(c): i for i, c in enumerate(np.asarray(coords).tolist())}
    return np.array([index[tuple(c)] for c in np.asarray(chosen).tolist()], np.int64)


def choose_subset(coords) -> np.ndarray:
    step = max(1, len(coords) // N_SUBSET)
    return np.asarray(coords)[::step][:N_SUBSET]


def oracle_states(L, O, depth_u16, rgb, poses):
    """The oracle's integration cases: frame A into an empty map (colour
    update), then frame B by the colour update and, from the same state, by
    the normal-weighted update with frame B's normal map.  Returns a dict of
    canonical states and the visible-block lists of both fuses."""
    K, cfg = intrinsics(L), config(L)
    fB = O.OracleFrame(O.config_from(cfg), O.intrinsics_from(K))
    fB.build(depth_m(depth_u16[1]), rgb[1])
    nmap_b = fB.get(1, 0)
    out = {"nmap_b": nmap_b}
    for mode in ("colour", "weighted"):
        om = O.OracleMap(O.config_from(cfg), O.intrinsics_from(K))
        om.fuse(depth_m(depth_u16[0]), rgb[0], poses[0])
        if mode == "colour":
            out["visible_a"] = om.visible()
            out["s1"] = map_state_from_oracle(*om.export())
            om.fuse(depth_m(depth_u16[1]), rgb[1], poses[1])
            out["visible_b"] = om.visible()
        else:
            om.fuse(depth_m(depth_u16[1]), rgb[1], poses[1], nmap=nmap_b)
        out[f"s2_{mode}"] = map_state_from_oracle(*om.export())
    return out


# ---------------------------------------------------------------- raycast

def raycast_poses(poses):
    """The fuse pose of frame B, and one 6 cm to its side and turned 3 degrees
    (a view the map was not fused from)."""
    T = np.asarray(poses[1], np.float64)
    a = np.deg2rad(3.0)
    Rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    T2 = T.copy()
    T2[:3, :3] = T[:3, :3] @ Rz
    T2[:3, 3] = T[:3, 3] + T[:3, :3] @ np.array([0.06, 0.0, 0.0])
    return T, T2


def oracle_raycasts(L, O, depth_u16, rgb, poses, ray_poses):
    """The map after the colour updates of A and B; for each pose the z-range
    grid (cells x 2: min, max) and the vertex map (NaN canonical)."""
    K, cfg = intrinsics(L), config(L)
    om = O.OracleMap(O.config_from(cfg), O.intrinsics_from(K))
    om.fuse(depth_m(depth_u16[0]), rgb[0], poses[0])
    om.fuse(depth_m(depth_u16[1]), rgb[1], poses[1])
    res = []
    for T in ray_poses:
        v = om.raycast(T)
        res.append((om.zrange().copy(), canonical_nan(v)))
    return om, res


# ---------------------------------------------------------------- rows

def oracle_frames(L, O, depth_u16, rgb):
    K, cfg = intrinsics(L), config(L)
    fr = []
    for i in range(2):
        f = O.OracleFrame(O.config_from(cfg), O.intrinsics_from(K))
        f.build(depth_m(depth_u16[i]), rgb[i])
        fr.append(f)
    return fr


def frame_digest(frames) -> str:
    return digest(*[canonical_nan(f.get(kind, lvl)) for f in frames for lvl in LEVELS for kind in range(5)])


def oracle_rows(O, ref, cur, level, T, stddev):
    """(ICP rows, photometric rows) of every reference pixel at `level`:
    29 floats each (the 28 products of the row's upper triangle, then the
    correspondence flag)."""
    t = O.reduce_terms(ref, cur, level, T, stddev)
    return np.ascontiguousarray(t[:, :29]), np.ascontiguousarray(t[:, 29:])


def sample_pixels(n_pixels: int, level: int) -> np.ndarray:
    rng = np.random.default_rng(1000 + level)
    return np.sort(rng.choice(n_pixels, size=min(N_SAMPLE, n_pixels), replace=False))


# ---------------------------------------------------------------- image kernels

def oracle_images(L, O, depth_u16, rgb):
    """Frame B's images at the pinned levels: the kernels' inputs (metric
    depth, intensity) and the oracle's outputs (vertex and normal maps,
    gradients)."""
    f = oracle_frames(L, O, depth_u16, rgb)[1]
    return {level: {"depth": f.get(5, level), "intensity": f.get(2, level), "vmap": canonical_nan(f.get(0, level)),
                    "nmap": canonical_nan(f.get(1, level)), "dx": f.get(3, level), "dy": f.get(4, level)}
            for level in LEVELS}


def interior(a: np.ndarray) -> np.ndarray:
    """All but the last row and column: computeDerivativeK and computeNMapK
    write nothing there (cuda_imgproc.cu:224, :280)."""
    return a[:-1, :-1]


def oracle_shading(O, depth_u16, rgb, images):
    """renderScene and renderSceneTextured of frame B's level-0 maps."""
    im = images[0]
    return O.render_scene(im["vmap"], im["nmap"]), O.render_scene(im["vmap"], im["nmap"], rgb[1])


# ---------------------------------------------------------------- marching cubes

def sort_triangles(v, *attrs):
    """Canonical order of a triangle soup: by the 9 vertex coordinates, ties by
    the attributes (NaN normals of degenerate triangles last)."""
    cols = [v.reshape(len(v), 9)[:, i] for i in range(9)]
    for a in attrs:
        flat = a.reshape(len(a), -1).astype(np.float64)
        cols += [np.nan_to_num(flat[:, i], nan=1e30) for i in range(flat.shape[1])]
    order = np.lexsort(cols[::-1])
    return (v[order],) + tuple(a[order] for a in attrs)


def oracle_meshes(om):
    """Marching cubes of a map: (vertices, normals) and (vertices, colours),
    each in canonical order, NaN canonical."""
    v1, n1 = om.mesh(1, 1 << 20)
    v2, c2 = om.mesh(2, 1 << 20)
    a = sort_triangles(v1, n1)
    b = sort_triangles(v2, c2)
    return (canonical_nan(a[0]), canonical_nan(a[1])), (canonical_nan(b[0]), b[1])


def sample_triangles(n: int) -> np.ndarray:
    rng = np.random.default_rng(77)
    return np.sort(rng.choice(n, size=min(1024, n), replace=False))
