"""gbf_reduce_noalloc: the ICP + photometric reduction for callers that cannot
allocate device memory -- code recording a CUDA graph (cudaMalloc cannot be
captured), real-time loops that forbid allocation after start-up, and
frameworks that hand out all device memory themselves.  It takes the images
and the output buffer from the caller and keeps its scratch in a fixed array
inside the library.  This file is collected last on purpose: it checks the
allocation-free entry point against the existing session-based gbf_reduce on
the same images, twice in a row (the second call reuses the shared scratch
the first one left behind)."""
import ctypes as C

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _inputs(L, K, cfg, imgs):
    ref_v, ref_n, ref_i, cur_v, cur_n, cur_i, cur_dx, cur_dy = imgs
    return L._lib.ReduceInputs(K.width, K.height, K.fx, K.fy, K.cx, K.cy,
                               ref_v.data_ptr(), ref_n.data_ptr(), ref_i.data_ptr(),
                               cur_v.data_ptr(), cur_n.data_ptr(), cur_i.data_ptr(),
                               cur_dx.data_ptr(), cur_dy.data_ptr(),
                               cfg.icp_dist_thresh, cfg.icp_angle_thresh)


def test_noalloc_reduce_matches_session_reduce(gbf):
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 0, bilateral=0)
    fr = H.frames(L, K, 2, step=1)
    t = L.DenseTracking(K, cfg)
    t.set_reference(H.cuda(H.depth_m(fr[0][0])), H.cuda(fr[0][1]))
    t.set_current(H.cuda(H.depth_m(fr[1][0])), H.cuda(fr[1][1]))
    # the session's level-0 images, copied into caller-owned buffers
    imgs = (t.get_image(1, 0, 0), t.get_image(1, 1, 0), t.get_image(1, 2, 0),
            t.get_image(0, 0, 0), t.get_image(0, 1, 0), t.get_image(0, 2, 0),
            t.get_image(0, 3, 0), t.get_image(0, 4, 0))
    inp = _inputs(L, K, cfg, imgs)
    rel = np.linalg.inv(fr[1][2]) @ fr[0][2]
    for T, sd in ((rel, 0.0), (rel, 6.0)):
        want = t.reduce(0, T, sd)
        assert want[28] > 100 and want[57] > 100
        scale = np.maximum(np.abs(want), 1e-3 * np.abs(want).max())
        for _ in range(2):  # two calls in a row share the scratch array
            out = torch.full((58,), float("nan"), dtype=torch.float64, device="cuda")
            L._lib.call("gbf_reduce_noalloc", C.byref(inp), L._lib.mat16(T), sd, out.data_ptr(),
                        torch.cuda.current_stream().cuda_stream)
            got = out.cpu().numpy()
            assert got[28] == want[28] and got[57] == want[57]
            assert np.all(np.abs(got - want) <= 2e-5 * scale + 1e-9)


def test_noalloc_reduce_rejects_oversized_images(gbf):
    import torch
    L = gbf
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    p = buf.data_ptr()
    inp = L._lib.ReduceInputs(4096, 1024, 500.0, 500.0, 2047.5, 511.5, p, p, p, p, p, p, p, p, 0.01, 0.866)
    out = torch.zeros(58, dtype=torch.float64, device="cuda")
    with pytest.raises(L.GbfError) as e:
        L._lib.call("gbf_reduce_noalloc", C.byref(inp), L._lib.mat16(np.eye(4)), 0.0, out.data_ptr(), 0)
    assert e.value.status == 4  # GBF_ERR_CAPACITY
