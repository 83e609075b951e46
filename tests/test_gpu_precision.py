"""Error of the GPU path against the FP64 oracle (double arithmetic,
unquantised voxel storage) and against the synthetic ground truth:

* TSDF error in units of the truncation distance, with ground-truth poses;
* raycast depth (camera z) at the last pose of the same fused map;
* marching-cubes mesh, symmetric Chamfer distance between the vertex sets;
* pose drift of the full tracking loop against the FP64 oracle;
* trajectory error (ATE / RPE) of the tracking loop against the ground truth.
"""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu

N_FUSE = 30
_FUSED = {}


def _fused(L, layout):
    """GPU map and FP64 oracle map after N_FUSE normal-weighted updates at the
    ground-truth poses (the System's fusion path), shared by the tests below."""
    if layout in _FUSED:
        return _FUSED[layout]
    import oracle as O
    K = H.intrinsics(L)
    cfg = H.small_config(L, layout)
    m = L.DenseMapping(K, cfg)
    o64 = O.OracleMap(O.config_from(cfg), O.intrinsics_from(K), "f64")
    o32 = O.OracleMap(O.config_from(cfg), O.intrinsics_from(K), "f32")
    fr = O.OracleFrame(O.config_from(cfg), O.intrinsics_from(K))
    frames = H.frames(L, K, N_FUSE, step=1)
    for d, c, T in frames:
        dm = H.depth_m(d)
        fr.build(dm, c)
        n0 = fr.get(1, 0)
        m.update(H.cuda(dm), H.cuda(c), T, normal=H.cuda(n0))
        o64.fuse(dm, c, T, nmap=n0)
        o32.fuse(dm, c, T, nmap=n0)
    _FUSED[layout] = (K, cfg, m, o64, frames[-1][2], o32)
    return _FUSED[layout]


def _common(gmap, omap):
    gc, gs, gw, _ = H.sort_blocks(*gmap)
    oc, os_, ow, _ = H.sort_blocks(*omap)
    gk = {tuple(c): i for i, c in enumerate(gc)}
    idx = [(gk[tuple(c)], j) for j, c in enumerate(oc) if tuple(c) in gk]
    gi = np.array([a for a, _ in idx])
    oi = np.array([b for _, b in idx])
    return gs[gi], gw[gi], os_[oi], ow[oi]


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_tsdf_error_vs_fp64_oracle(gbf, layout):
    K, cfg, m, o64, _, o32 = _fused(gbf, layout)
    gmap = m.export()
    gs, gw, os_, ow = _common(gmap, o64.export())
    both = (gw > 0) & (ow > 0)
    err = np.abs(gs[both] - os_[both])   # sdf is stored in units of the truncation distance
    p999 = float(np.quantile(err, 0.999))
    # the same error split in two: the kernels and the layout's storage against
    # the FP32 oracle (the reference's arithmetic in the layout's storage), and
    # that FP32 arithmetic itself against FP64
    gs2, gw2, fs, fw = _common(gmap, o32.export())
    impl = np.abs(gs2[(gw2 > 0) & (fw > 0)] - fs[(gw2 > 0) & (fw > 0)])
    fs3, fw3, os3, ow3 = _common(o32.export(), o64.export())
    arith = np.abs(fs3[(fw3 > 0) & (ow3 > 0)] - os3[(fw3 > 0) & (ow3 > 0)])
    print(f"layout {layout}: voxels {both.sum()}, TSDF |err|/tau max {err.max():.2e} p99.9 {p999:.2e} "
          f"mean {err.mean():.2e}; GPU vs FP32 oracle max {impl.max():.2e}; FP32 oracle vs FP64 max "
          f"{arith.max():.2e} p99.9 {np.quantile(arith, 0.999):.2e}, above 1e-3: GPU {np.sum(err > 1e-3)} "
          f"FP32 oracle {np.sum(arith > 1e-3)}")
    # The maximum comes from the reference's FP32 arithmetic, not from this
    # implementation: the FP32 oracle is as far from FP64 at its worst voxel, and
    # the GPU stays within a few storage steps of the FP32 oracle everywhere
    # (sinf rounds differently in CUDA and libm; HALF's fp16 step near 1 is 4.9e-4).
    assert impl.max() <= (4e-3 if layout == 1 else 5e-4)
    assert abs(err.max() - arith.max()) <= impl.max()
    # FP32 and FP64 can pick a different depth pixel for a voxel on a pixel
    # boundary, so the bound is on the distribution.  REF (int16 sdf, 3e-5
    # quantum, truncating) and SNORM (the same quantum, rounded to nearest):
    # 99.9 % of the voxels within 1e-3 of the truncation distance.  HALF (fp16
    # sdf, 2.4e-4 rounding near +-1, re-rounded every update): the tail is
    # wider; measured p99.9 1.5e-3, mean 1.4e-4.
    assert p999 <= (2e-3 if layout == 1 else 1e-3)
    assert err.mean() < 2e-4


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_raycast_depth_vs_fp64_oracle(gbf, layout):
    """Raycast of the fused map at the last pose: camera-space depth against the
    FP64 oracle's raycast of its FP64 map.  A ray that passes a thin gap or a
    grazing surface can stop on a different surface in FP32 than in FP64 (a
    difference of metres on one ray), so the depth RMS is taken over the rays
    that hit the same surface (|dz| < truncation distance) and the others are
    counted and bounded separately."""
    import torch
    L = gbf
    K, cfg, m, o64, T, _ = _fused(L, layout)
    vm = torch.full((K.height, K.width, 4), float("nan"), device="cuda")
    m.raycast(vm, T)
    g = vm.cpu().numpy()
    o = o64.raycast(T)
    gh, oh = ~np.isnan(g[..., 2]), ~np.isnan(o[..., 2])
    both = gh & oh
    dz = np.abs(g[..., 2][both] - o[..., 2][both]).astype(np.float64)
    same = dz < cfg.truncation
    rms = float(np.sqrt(np.mean(dz[same] ** 2)))
    print(f"layout {layout}: rays hit {gh.sum()} (FP64 {oh.sum()}), hit masks differ on {np.sum(gh != oh)}, "
          f"other surface {np.sum(~same)}; same-surface depth RMS {rms * 1e3:.4f} mm, "
          f"p99 {np.quantile(dz[same], 0.99) * 1e3:.4f} mm, max {dz[same].max() * 1e3:.3f} mm")
    assert gh.mean() > 0.8
    assert np.sum(gh != oh) <= 1e-3 * both.sum()
    assert np.sum(~same) <= 1e-3 * both.sum()
    # measured RMS 0.05 (SNORM) - 0.12 (HALF) mm, p99 11-24 um: a few grazing
    # rays, where a small sdf difference moves the zero crossing far along the
    # ray, dominate the RMS
    assert rms < 0.25e-3
    assert np.quantile(dz[same], 0.99) < 0.05e-3


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_mesh_chamfer_vs_fp64_oracle(gbf, layout):
    """Marching cubes of the fused map against the FP64 oracle's mesh of its
    FP64 map: symmetric Chamfer distance (mean of the two nearest-neighbour
    means) between the triangle vertex sets."""
    import torch
    spatial = pytest.importorskip("scipy.spatial")
    L = gbf
    K, cfg, m, o64, _, _ = _fused(L, layout)
    ov, _ = o64.mesh(0, 1 << 22)
    cap = len(ov) + (1 << 16)
    vtx = torch.zeros((cap, 3, 3), dtype=torch.float32, device="cuda")
    n = m.fetch_mesh_vertex_only(vtx)
    assert 0 < n < cap
    gp = vtx[:n].cpu().numpy().reshape(-1, 3).astype(np.float64)
    op = ov.reshape(-1, 3).astype(np.float64)
    d_go, _ = spatial.cKDTree(op).query(gp)
    d_og, _ = spatial.cKDTree(gp).query(op)
    chamfer = 0.5 * (d_go.mean() + d_og.mean())
    print(f"layout {layout}: triangles {n} (FP64 {len(ov)}), Chamfer {chamfer * 1e3:.4f} mm, "
          f"p99 {max(np.quantile(d_go, 0.99), np.quantile(d_og, 0.99)) * 1e3:.4f} mm, "
          f"Hausdorff {max(d_go.max(), d_og.max()) * 1e3:.3f} mm")
    assert abs(n - len(ov)) <= 1e-3 * len(ov)
    assert chamfer < 0.05e-3  # 50 um at a 1 cm voxel; CPU estimate of this case 2-4 um


def test_pose_drift_vs_fp64_oracle(gbf):
    import oracle as O
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    fr = H.frames(L, K, 30)
    s = L.System(K, cfg)
    s.set_pose(fr[0][2])
    o64 = O.OracleSystem(O.config_from(cfg), O.intrinsics_from(K), "f64")
    o64.set_pose(fr[0][2])
    drift = []
    for d, c, T in fr:
        s.process_images(H.cuda(d), H.cuda(c))
        o64.process(d, c)
        drift.append(np.abs(s.get_camera_pose()[:3, 3] - o64.pose()[:3, 3]).max())
    print(f"pose drift vs FP64 oracle over {len(fr)} frames: max {max(drift)*1e3:.3f} mm")
    assert max(drift) < 1e-3  # the target bound: 1 mm


def _rel(a, b):
    return np.linalg.inv(a) @ b


@pytest.mark.parametrize("layout", [1, 2])
def test_trajectory_error_vs_ground_truth(gbf, layout):
    """Tracking loop over 100 frames of the synthetic circle trajectory, started
    at the ground-truth pose: absolute trajectory error (RMS of the camera
    position error; no alignment needed, both start at the same pose) and
    relative pose error over one frame (RMS of the translation and rotation of
    (gt_k^-1 gt_k+1)^-1 (est_k^-1 est_k+1))."""
    L = gbf
    K = H.intrinsics(L)
    s = L.System(K, H.small_config(L, layout))
    fr = H.frames(L, K, 100)
    s.set_pose(fr[0][2])
    est = []
    for d, c, T in fr:
        s.process_images(H.cuda(d), H.cuda(c))
        est.append(s.get_camera_pose())
    gt = [np.asarray(T, np.float64) for _, _, T in fr]
    ate = np.sqrt(np.mean([np.sum((e[:3, 3] - g[:3, 3]) ** 2) for e, g in zip(est, gt)]))
    rpe_t, rpe_r = [], []
    for k in range(len(gt) - 1):
        E = _rel(_rel(gt[k], gt[k + 1]), _rel(est[k], est[k + 1]))
        rpe_t.append(np.sum(E[:3, 3] ** 2))
        rpe_r.append(np.arccos(np.clip((np.trace(E[:3, :3]) - 1) / 2, -1, 1)) ** 2)
    rpe_t = np.sqrt(np.mean(rpe_t))
    rpe_r = np.degrees(np.sqrt(np.mean(rpe_r)))
    print(f"layout {layout}: ATE RMS {ate * 1e3:.2f} mm over {len(gt)} frames, RPE {rpe_t * 1e3:.3f} mm / "
          f"{rpe_r:.4f} deg per frame")
    # measured at 320x240 with the depth noise model: ATE 4.8 mm, RPE 0.35 mm mean
    assert ate < 0.01
    assert rpe_t < 1e-3
