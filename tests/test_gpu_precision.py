"""Error of the GPU path against the FP64 oracle (double arithmetic,
unquantised voxel storage): TSDF max-abs in units of the truncation distance
with ground-truth poses, and pose drift of the full tracking loop."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


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
    import oracle as O
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, layout)
    m = L.DenseMapping(K, cfg)
    o64 = O.OracleMap(O.config_from(cfg), O.intrinsics_from(K), "f64")
    fr = O.OracleFrame(O.config_from(cfg), O.intrinsics_from(K))
    for d, c, T in H.frames(L, K, 30, step=1):
        dm = H.depth_m(d)
        fr.build(dm, c)
        n0 = fr.get(1, 0)
        m.update(H.cuda(dm), H.cuda(c), T, normal=H.cuda(n0))
        o64.fuse(dm, c, T, nmap=n0)
    gs, gw, os_, ow = _common(m.export(), o64.export())
    both = (gw > 0) & (ow > 0)
    err = np.abs(gs[both] - os_[both])   # sdf is stored in units of the truncation distance
    p999 = float(np.quantile(err, 0.999))
    print(f"layout {layout}: voxels {both.sum()}, TSDF |err|/tau max {err.max():.2e} p99.9 {p999:.2e} "
          f"mean {err.mean():.2e}")
    # FP32 and FP64 can pick a different depth pixel for a voxel on a pixel
    # boundary, so the bound is on the distribution.  REF (int16 sdf, 3e-5
    # quantum, truncating) and SNORM (the same quantum, rounded to nearest):
    # 99.9 % of the voxels within 1e-3 of the truncation distance.  HALF (fp16
    # sdf, 2.4e-4 rounding near +-1, re-rounded every update): the tail is
    # wider; measured p99.9 1.5e-3, mean 1.4e-4.
    assert p999 <= (2e-3 if layout == 1 else 1e-3)
    assert err.mean() < 2e-4


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
