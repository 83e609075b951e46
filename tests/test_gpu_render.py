"""The "next" rows around the per-frame path: a raycast from an arbitrary pose
with its own visibility pass (DenseMapping::raycast_check_visibility,
src/voxel_hashing/voxel_hashing.cpp:121-135) and headless Phong shading
(renderScene / renderSceneTextured, src/tracking/cuda_imgproc.cu:17-108), both
against the oracle."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _oracle_map(L, cfg, K):
    import oracle as O
    return O.OracleMap(O.config_from(cfg), O.intrinsics_from(K))


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_raycast_check_visibility_bit_exact(gbf, layout):
    """Fuse along the trajectory, then raycast from a pose the last fuse did not
    see from: the visible list is rebuilt for that pose on both sides."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, layout)
    m = L.DenseMapping(K, cfg)
    om = _oracle_map(L, cfg, K)
    fr = H.frames(L, K, 6, step=5)
    for d, c, T in fr:
        dm = H.depth_m(d)
        m.update(H.cuda(dm), H.cuda(c), T)
        om.fuse(dm, c, T)
    for T in (fr[1][2], fr[3][2]):
        vm = torch.full((K.height, K.width, 4), float("nan"), device="cuda")
        m.raycast_check_visibility(vm, T)
        g = vm.cpu().numpy()
        o = om.raycast_check_visibility(T)
        vg = {tuple(x) for x in m.visible_blocks()}
        vo = {tuple(x) for x in om.visible()}
        assert vg == vo, f"visible sets differ: {len(vg ^ vo)} blocks"
        assert np.array_equal(m.zrange(), om.zrange()), "z-range grids differ"
        gh, oh = ~np.isnan(g[..., 2]), ~np.isnan(o[..., 2])
        assert np.array_equal(gh, oh), f"hit masks differ in {np.sum(gh != oh)} pixels"
        assert gh.mean() > 0.8
        assert np.array_equal(g[gh], o[oh])


def _device_pow20(x):
    """CUDA's powf(x, 20.f) of float32 arguments (a float32 tensor-tensor pow)."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    return torch.pow(t, torch.full_like(t, 20.0)).cpu().numpy()


def test_render_scene_matches_oracle(gbf):
    """Shaded model prediction of a System session, plain and textured, bit for
    bit: every step rounds as written on both sides, and the oracle takes
    CUDA's powf(x, 20) for the bases it evaluates (recorded in a first run).
    With libm's powf instead, a truncated 8-bit value may move by one on rare
    pixels, which the second check bounds."""
    import oracle as O
    import torch
    L = gbf
    K = H.intrinsics(L)
    s = L.System(K, H.small_config(L, 0))
    fr = H.frames(L, K, 3, step=3)
    s.set_pose(fr[0][2])
    for d, c, _ in fr:
        s.process_images(H.cuda(d), H.cuda(c))
    torch.cuda.synchronize()
    vm = s.get_image(1, 0, 0)  # model prediction: vertex / normal maps of the reference set
    nm = s.get_image(1, 1, 0)
    v, n = vm.cpu().numpy(), nm.cpu().numpy()
    assert np.isfinite(v[..., 2]).mean() > 0.8
    rgb = fr[-1][1]
    for textured in (False, True):
        g = (s.get_rendered_scene_textured() if textured else s.get_rendered_image()).cpu().numpy()
        exact, sizes, misses = O.with_device_transcendentals(
            lambda: O.render_scene(v, n, rgb if textured else None), {O.TRANS_POW20: _device_pow20})
        assert sizes[O.TRANS_POW20] > 1000 and misses[O.TRANS_POW20] == 0
        assert np.array_equal(g, exact)
        o = O.render_scene(v, n, rgb if textured else None)
        diff = np.abs(g.astype(np.int32) - o.astype(np.int32))
        assert diff.max() <= 1
        assert (diff > 0).mean() < 2e-3
        assert (g[..., 3] == 255).all()
        # the free function on the same maps gives the session's image
        f = L.render_scene(vm, nm, H.cuda(rgb) if textured else None).cpu().numpy()
        assert np.array_equal(f, g)
    # background colour where the prediction is empty
    bg = np.isnan(v[..., 0])
    if bg.any():
        assert (g[bg][:, :3] == O.render_scene(np.full((1, 1, 4), np.nan, np.float32),
                                               np.zeros((1, 1, 4), np.float32))[0, 0, :3]).all()
