"""gbf_reduce_noalloc: the ICP + photometric reduction for callers that cannot
allocate device memory -- real-time loops that forbid allocation once they run,
and frameworks that hand out all device memory through their own allocator.
It takes the images and the output buffer from the caller and keeps its
scratch in a fixed array inside the library.

This file is collected last on purpose.  It checks the allocation-free entry
point against the session-based gbf_reduce on the same images (the same
per-CTA partials added in the same order, so bit for bit) and against the
oracle, twice in a row each time (the second call reuses the shared scratch
the first one left behind), at the largest image the scratch holds and at a
pixel count that is not a multiple of 4, with the images packed back to back
in one buffer."""
import ctypes as C

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu

LIMIT_PIXELS = 2048 * 1024  # the fixed scratch holds 2048 CTAs of 1024 pixels


def _inputs(L, K, cfg, ptrs):
    return L._lib.ReduceInputs(K.width, K.height, K.fx, K.fy, K.cx, K.cy, *ptrs,
                               cfg.icp_dist_thresh, cfg.icp_angle_thresh)


def _noalloc(L, inp, T, sd):
    import torch
    out = torch.full((58,), float("nan"), dtype=torch.float64, device="cuda")
    L._lib.call("gbf_reduce_noalloc", C.byref(inp), L._lib.mat16(T), sd, out.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    return out.cpu().numpy()


def _session_images(t):
    # level 0 of the reference (set 1) and the current (set 0) frame, copied
    # into caller-owned buffers: vmap, nmap, intensity; vmap, nmap, I, dI/dx, dI/dy
    return (t.get_image(1, 0, 0), t.get_image(1, 1, 0), t.get_image(1, 2, 0),
            t.get_image(0, 0, 0), t.get_image(0, 1, 0), t.get_image(0, 2, 0),
            t.get_image(0, 3, 0), t.get_image(0, 4, 0))


def _oracle_pair(L, K, cfg, a, b):
    import oracle as O
    ref = O.OracleFrame(O.config_from(cfg), O.intrinsics_from(K))
    cur = O.OracleFrame(O.config_from(cfg), O.intrinsics_from(K))
    ref.build(H.depth_m(a[0]), a[1])
    cur.build(H.depth_m(b[0]), b[1])
    return ref, cur


def _close_to_oracle(got, o):
    assert got[28] == o[28] and got[57] == o[57], "correspondence counts differ from the oracle's"
    scale = np.maximum(np.abs(o), 1e-3 * np.abs(o).max())
    # FP32 tree + compensated partial sums against the oracle's FP64 sequential sums
    assert np.all(np.abs(got - o) <= 2e-5 * scale + 1e-9), float(np.max(np.abs(got - o) / scale))


def _check_against_session(L, K, cfg):
    import oracle as O
    fr = H.frames(L, K, 2, step=1)
    t = L.DenseTracking(K, cfg)
    t.set_reference(H.cuda(H.depth_m(fr[0][0])), H.cuda(fr[0][1]))
    t.set_current(H.cuda(H.depth_m(fr[1][0])), H.cuda(fr[1][1]))
    imgs = _session_images(t)
    inp = _inputs(L, K, cfg, [x.data_ptr() for x in imgs])
    ref, cur = _oracle_pair(L, K, cfg, fr[0], fr[1])
    rel = np.linalg.inv(fr[1][2]) @ fr[0][2]
    for T, sd in ((rel, 0.0), (rel, 6.0)):
        want = t.reduce(0, T, sd)
        assert want[28] > 100 and want[57] > 100
        o = O.reduce(ref, cur, 0, T, sd)
        for _ in range(2):  # two calls in a row share the scratch array
            got = _noalloc(L, inp, T, sd)
            assert np.array_equal(got, want), "differs from gbf_reduce on the same images"
            _close_to_oracle(got, o)


def test_noalloc_reduce_matches_session_reduce(gbf):
    L = gbf
    _check_against_session(L, H.intrinsics(L), H.small_config(L, 0, bilateral=0))


def test_noalloc_reduce_at_the_pixel_limit(gbf):
    """2048 x 1024 = 2,097,152 pixels: every one of the scratch's 2048 partial
    records in use."""
    L = gbf
    K = L.IntrinsicMatrix(2048, 1024, 1680.0, 1680.0, 1023.5, 511.5)
    assert K.width * K.height == LIMIT_PIXELS
    _check_against_session(L, K, H.small_config(L, 0, bilateral=0, num_blocks=1 << 12, num_buckets=1 << 13))


def test_noalloc_reduce_odd_pixel_count_tight_buffer(gbf):
    """321 x 241 pixels (not a multiple of 4) from the oracle's level-0 images,
    packed back to back in one device buffer with the reference intensity at
    its very end."""
    import oracle as O
    import torch
    L = gbf
    K = L.IntrinsicMatrix(321, 241, 263.0, 263.0, 160.0, 120.0)
    P = K.width * K.height
    assert P % 4 != 0
    cfg = H.small_config(L, 0, bilateral=0, num_levels=1)
    fr = H.frames(L, K, 2, step=1)
    ref, cur = _oracle_pair(L, K, cfg, fr[0], fr[1])
    parts = [ref.get(0, 0), ref.get(1, 0), cur.get(0, 0), cur.get(1, 0), cur.get(2, 0), cur.get(3, 0),
             cur.get(4, 0)]
    ref_i = ref.get(2, 0).reshape(-1)
    off, offs = 0, []
    for a in parts:
        offs.append(off)
        off += a.size
    off = (off + 3) // 4 * 4  # the reference intensity starts on a 16-byte boundary
    buf = np.zeros(off + P, np.float32)
    for o, a in zip(offs, parts):
        buf[o:o + a.size] = a.reshape(-1)
    buf[off:] = ref_i
    dev = H.cuda(buf)
    base, f = dev.data_ptr(), 4
    rv, rn, cv, cn, ci, cdx, cdy = (base + f * o for o in offs)
    inp = _inputs(L, K, cfg, [rv, rn, base + f * off, cv, cn, ci, cdx, cdy])
    rel = np.linalg.inv(fr[1][2]) @ fr[0][2]
    torch.cuda.synchronize()
    for T, sd in ((np.eye(4), 0.0), (rel, 6.0)):
        o = O.reduce(ref, cur, 0, T, sd)
        assert o[28] > 100 and o[57] > 100
        first = _noalloc(L, inp, T, sd)
        second = _noalloc(L, inp, T, sd)
        assert np.array_equal(first, second)
        _close_to_oracle(first, o)


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


def test_noalloc_reduce_rejects_misaligned_output(gbf):
    """The sums are written as doubles: an output pointer off an 8-byte
    boundary is refused on the host, before anything is launched."""
    import torch
    L = gbf
    buf = torch.zeros(1024, dtype=torch.float32, device="cuda")
    p = buf.data_ptr()
    inp = L._lib.ReduceInputs(64, 64, 50.0, 50.0, 31.5, 31.5, p, p, p, p, p, p, p, p, 0.01, 0.866)
    out = torch.zeros(60, dtype=torch.float64, device="cuda")
    with pytest.raises(L.GbfError) as e:
        L._lib.call("gbf_reduce_noalloc", C.byref(inp), L._lib.mat16(np.eye(4)), 0.0, out.data_ptr() + 4, 0)
    assert e.value.status == 1  # GBF_ERR_INVALID_ARG
