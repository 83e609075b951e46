"""The oracle, and the CUDA kernels, against outputs of the reference's own
kernels.

tests/golden/ref_kernels.npz holds what the reference's integration
(update_map_with_colour_kernel, update_map_weighted_kernel:
src/voxel_hashing/depth_fusion.cu:288-428), z-range tiles
(RenderingBlockDelegate, ray_tracing.cu:17-277), raycast march
(MapRenderingDelegate::operator(), ray_tracing.cu:346-425), ICP row
(ICPReduction::getRow, src/tracking/pose_estimator.cu:166-222), photometric
row (RgbReduction2::compute_jacobian, m_estimator.cu:313-391), image kernels
(computeDerivativeK, backProjectDepthK, computeNMapK, renderSceneK,
renderSceneTexturedK: src/tracking/cuda_imgproc.cu:17-305) and marching cubes
(BuildVertexArray, BuildVertexAndColourArray: src/voxel_hashing/
scene_mesh.cu:14-643) computed on a GB300 from the reference sources, built
with every float operation rounded as written
(tests/golden/make_kernel_golden.py; cases in tests/golden/pin_cases.py).

CPU tests: the oracle recomputes every case from the stored frames.  Integer
and float results are compared bit for bit.  The normal-weighted update's
weight |sin(n_z)| / d^2 takes CUDA's sinf in the reference and libm's in the
oracle (a few ulp apart): with the fixture's table of CUDA's sinf for the
arguments the oracle evaluates it matches bit for bit too; with libm's sinf the
sdf codes may differ by one truncation step and the colours by one level, on
a small share of the voxels.

GPU tests: the CUDA kernels on the same inputs match the reference's outputs
bit for bit, the normal-weighted update included (both use CUDA's sinf), and
so do the marching cubes and the shading (CUDA's powf on both sides).
"""
from pathlib import Path
import sys

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
import pin_cases as P  # noqa: E402

FIX = ROOT / "tests" / "golden" / "ref_kernels.npz"


@pytest.fixture(scope="module")
def fx():
    return np.load(FIX)


@pytest.fixture(scope="module")
def lib():
    from libfusion_gb300 import build as B
    B.build()
    import libfusion_gb300 as L
    L.lib()
    return L


@pytest.fixture(scope="module")
def oracle_mod(oracle_lib):
    import oracle as O
    return O


def frames(fx):
    return fx["depth_u16"], fx["rgb"], fx["poses"]


def test_derived_inputs_are_the_ones_the_reference_saw(fx, lib, oracle_mod):
    """The oracle rebuilds, bit for bit, the vertex, normal, intensity and
    gradient images the reference kernels were given."""
    d, c, _ = frames(fx)
    assert P.frame_digest(P.oracle_frames(lib, oracle_mod, d, c)) == str(fx["frame_digest"])


@pytest.fixture(scope="module")
def states(fx, lib, oracle_mod):
    return P.oracle_states(lib, oracle_mod, *frames(fx))


@pytest.mark.parametrize("case", ["s1", "s2_colour"])
def test_colour_integration_bit_exact(fx, states, case):
    coords, code, w, rgb = states[case]
    assert np.array_equal(coords, fx[f"{case}_coords"]), "allocated block sets differ"
    idx = P.subset_rows(coords, fx[f"{case}_subset"])
    assert np.array_equal(code[idx], fx[f"{case}_subset_code"])
    assert np.array_equal(w[idx].view(np.int32), fx[f"{case}_subset_weight"].view(np.int32))
    assert np.array_equal(rgb[idx], fx[f"{case}_subset_rgb"])
    assert P.digest(coords, code, w, rgb) == str(fx[f"{case}_digest"]), "voxels outside the stored subset differ"


def test_weighted_integration_bit_exact_with_device_sinf(fx, lib, oracle_mod):
    """With CUDA's sinf values for the arguments it evaluates (stored in the
    fixture by its generator), the oracle's normal-weighted update equals the
    reference kernel's output bit for bit."""
    O = oracle_mod
    assert len(fx["sin_x"]) > 1000
    O.trans_table(O.TRANS_SIN, fx["sin_x"], fx["sin_y"])
    try:
        st = P.oracle_states(lib, O, *frames(fx))
        misses = O.trans_misses(O.TRANS_SIN)
    finally:
        O.trans_table(O.TRANS_SIN)
    assert misses == 0, "an argument the generator did not record"
    coords, code, w, rgb = st["s2_weighted"]
    assert np.array_equal(coords, fx["s2_weighted_coords"])
    idx = P.subset_rows(coords, fx["s2_weighted_subset"])
    assert np.array_equal(code[idx], fx["s2_weighted_subset_code"])
    assert np.array_equal(w[idx].view(np.int32), fx["s2_weighted_subset_weight"].view(np.int32))
    assert np.array_equal(rgb[idx], fx["s2_weighted_subset_rgb"])
    assert P.digest(coords, code, w, rgb) == str(fx["s2_weighted_digest"]), "voxels outside the stored subset differ"


def test_weighted_integration_within_sinf_rounding(fx, states):
    coords, code, w, rgb = states["s2_weighted"]
    assert np.array_equal(coords, fx["s2_weighted_coords"])
    idx = P.subset_rows(coords, fx["s2_weighted_subset"])
    rc, rw, rr = fx["s2_weighted_subset_code"], fx["s2_weighted_subset_weight"], fx["s2_weighted_subset_rgb"]
    gc, gw, gr = code[idx], w[idx], rgb[idx]
    assert np.array_equal(gw == 0, rw == 0), "observed voxels differ"
    # weight: one float rounding of sin apart, carried through the running sum
    assert np.all(np.abs(gw - rw) <= 4e-6 * np.maximum(np.abs(rw), 1e-30))
    # sdf code: truncating pack of a running mean that moved by ulps
    assert np.abs(gc.astype(int) - rc.astype(int)).max() <= 1
    assert np.abs(gr.astype(int) - rr.astype(int)).max() <= 1
    assert np.mean(gc != rc) < 0.01 and np.mean(np.any(gr != rr, axis=-1)) < 0.01


@pytest.fixture(scope="module")
def rays(fx, lib, oracle_mod):
    d, c, poses = frames(fx)
    return P.oracle_raycasts(lib, oracle_mod, d, c, poses, P.raycast_poses(poses))[1]


@pytest.mark.parametrize("k", [0, 1])
def test_zrange_and_raycast_bit_exact(fx, rays, k):
    z, v = rays[k]
    assert np.array_equal(z.view(np.int32), fx[f"zrange_{k}"].view(np.int32)), "z-range grids differ"
    ref = fx[f"vmap_{k}"]
    assert np.isfinite(ref[..., 2]).mean() > 0.5
    assert np.array_equal(v.view(np.int32), ref.view(np.int32)), "vertex maps differ"


@pytest.fixture(scope="module")
def rows(fx, lib, oracle_mod):
    d, c, poses = frames(fx)
    fr = P.oracle_frames(lib, oracle_mod, d, c)
    T = P.relative(poses[0], poses[1])
    out = {}
    for level in P.LEVELS:
        for sd in P.STDDEVS:
            icp, pho = P.oracle_rows(oracle_mod, fr[0], fr[1], level, T, sd)
            out[f"icp_{level}"] = icp
            out[f"rgb_{level}_{sd:g}"] = pho
    return out


@pytest.mark.parametrize("case", [f"icp_{l}" for l in P.LEVELS] +
                         [f"rgb_{l}_{sd:g}" for l in P.LEVELS for sd in P.STDDEVS])
def test_rows_bit_exact(fx, rows, case):
    got = rows[case]
    n = len(got)
    assert n == (P.W >> int(case.split("_")[1])) * (P.H >> int(case.split("_")[1]))
    found = np.unpackbits(fx[f"{case}_found"])[:n].astype(bool)
    assert found.sum() >= 200  # a case with correspondences to pin
    assert np.array_equal(got[:, 28] != 0, found), "correspondence sets differ"
    s = P.sample_pixels(n, int(case.split("_")[1]))
    assert np.array_equal(got[s].view(np.int32), fx[f"{case}_sample"].view(np.int32))
    assert P.digest(got) == str(fx[f"{case}_digest"]), "rows outside the stored sample differ"


# ------------------------------------------------------------------ the GPU kernels


def _gpu_map(L, fx, nmap=None):
    import torch
    d, c, poses = frames(fx)
    m = L.DenseMapping(P.intrinsics(L), P.config(L))
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    m.update(cu(P.depth_m(d[0])), cu(c[0]), poses[0])
    m.update(cu(P.depth_m(d[1])), cu(c[1]), poses[1], normal=None if nmap is None else cu(nmap))
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["colour", "weighted"])
def test_gpu_integration_matches_reference_kernels(gbf, fx, states, mode):
    L = gbf
    m = _gpu_map(L, fx, states["nmap_b"] if mode == "weighted" else None)
    coords, code, w, rgb = P.map_state_from_oracle(*m.export())
    key = f"s2_{mode}"
    assert np.array_equal(coords, fx[f"{key}_coords"])
    assert P.digest(coords, code, w, rgb) == str(fx[f"{key}_digest"])


@pytest.mark.gpu
def test_gpu_raycast_matches_reference_kernels(gbf, fx):
    import torch
    L = gbf
    m = _gpu_map(L, fx)
    for k, T in enumerate(P.raycast_poses(fx["poses"])):
        vm = torch.empty((P.H, P.W, 4), dtype=torch.float32, device="cuda")
        m.raycast(vm, T)
        v = P.canonical_nan(vm.cpu().numpy())
        assert np.array_equal(v.view(np.int32), fx[f"vmap_{k}"].view(np.int32)), k


# ------------------------------------------------------------------ image kernels, shading, marching cubes


@pytest.fixture(scope="module")
def images(fx, lib, oracle_mod):
    d, c, _ = frames(fx)
    return P.oracle_images(lib, oracle_mod, d, c)


@pytest.mark.parametrize("level", P.LEVELS)
def test_image_kernels_bit_exact(fx, images, level):
    """backProjectDepthK, computeNMapK and computeDerivativeK
    (src/tracking/cuda_imgproc.cu:217-305) on the oracle's level-`level`
    depth and intensity.  The reference leaves the last row and column of
    the normal and gradient maps unwritten; there the oracle writes NaN
    normals and zero gradients."""
    im = images[level]
    assert P.digest(im["vmap"]) == str(fx[f"img_vmap_{level}_digest"])
    assert P.digest(P.interior(im["nmap"])) == str(fx[f"img_nmap_{level}_digest"])
    assert bool(fx[f"img_nmap_{level}_border_unwritten"])
    for k in ("dx", "dy"):
        ref = fx[f"img_{k}_{level}"]
        assert np.array_equal(P.interior(im[k]).view(np.int32), P.interior(ref).view(np.int32)), k
        assert np.all(ref[-1] == 12345.0) and np.all(ref[:, -1] == 12345.0)  # unwritten by the reference


def test_shading_matches_reference(fx, images):
    """renderSceneK / renderSceneTexturedK (cuda_imgproc.cu:17-108): the
    specular term takes CUDA's powf in the reference and libm's in the
    oracle, so a channel may differ by one level on a few pixels; on this
    frame none does."""
    d, c, _ = frames(fx)
    import oracle as O
    plain, textured = P.oracle_shading(O, d, c, images)
    for got, key in ((plain, "shade"), (textured, "shade_textured")):
        diff = np.abs(got.astype(int) - fx[key].astype(int))
        assert diff.max() <= 1 and np.mean(diff.max(axis=-1) > 0) < 2e-3, key


@pytest.fixture(scope="module")
def meshes(fx, lib, oracle_mod):
    d, c, poses = frames(fx)
    om, _ = P.oracle_raycasts(lib, oracle_mod, d, c, poses, ())
    return P.oracle_meshes(om)


@pytest.mark.parametrize("kind", ["normal", "colour"])
def test_marching_cubes_bit_exact(fx, meshes, kind):
    """create_mesh_with_normal / create_mesh_with_colour (src/voxel_hashing/
    scene_mesh.cu:14-643) of the map after frames A and B, as triangle sets
    (the reference appends triangles in atomic order)."""
    v, a = meshes[0] if kind == "normal" else meshes[1]
    assert len(v) == int(fx[f"mesh_{kind}_count"]) and len(v) > 50000
    s = P.sample_triangles(len(v))
    assert np.array_equal(v[s].view(np.int32), fx[f"mesh_{kind}_sample_v"].view(np.int32))
    assert np.array_equal(a[s].view(np.int32 if kind == "normal" else np.uint8), fx[f"mesh_{kind}_sample_a"].view(
        np.int32 if kind == "normal" else np.uint8))
    assert P.digest(v, a) == str(fx[f"mesh_{kind}_digest"])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["normal", "colour"])
def test_gpu_marching_cubes_matches_reference_kernels(gbf, fx, kind):
    import torch
    L = gbf
    m = _gpu_map(L, fx)
    cap = int(fx[f"mesh_{kind}_count"]) + 64
    vtx = torch.zeros((cap, 3, 3), dtype=torch.float32, device="cuda")
    if kind == "normal":
        attr = torch.zeros((cap, 3, 3), dtype=torch.float32, device="cuda")
        n = m.fetch_mesh_with_normal(vtx, attr)
    else:
        attr = torch.zeros((cap, 3, 3), dtype=torch.uint8, device="cuda")
        n = m.fetch_mesh_with_colour(vtx, attr)
    assert n == int(fx[f"mesh_{kind}_count"])
    v, a = P.sort_triangles(vtx[:n].cpu().numpy(), attr[:n].cpu().numpy())
    v = P.canonical_nan(v)
    a = P.canonical_nan(a) if kind == "normal" else a
    assert P.digest(v, a) == str(fx[f"mesh_{kind}_digest"])


@pytest.mark.gpu
def test_gpu_shading_matches_reference_kernels(gbf, fx, images):
    L = gbf
    im = images[0]
    _, c, _ = frames(fx)
    plain = L.render_scene(H_cuda(im["vmap"]), H_cuda(im["nmap"])).cpu().numpy()
    textured = L.render_scene(H_cuda(im["vmap"]), H_cuda(im["nmap"]), H_cuda(c[1])).cpu().numpy()
    assert np.array_equal(plain, fx["shade"]) and np.array_equal(textured, fx["shade_textured"])


def H_cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()
