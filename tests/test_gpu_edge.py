"""Edge cases and failure paths on the GPU, injected from the host: exhausted
pools and tables (the reference drops blocks silently, map_struct.cu:205-223,
305-323), empty and invalid frames, lost tracking."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def test_pool_exhaustion_is_reported(gbf):
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 0, num_blocks=64))
    d, c, T = H.frames(L, K, 1)[0]
    m.update(H.cuda(H.depth_m(d)), H.cuda(c), T)
    st = m.stats()
    assert st.status & L.FLAG_POOL_EXHAUSTED
    assert st.allocated_blocks == 64
    coords = m.export()[0]
    assert len(coords) == 64 and len({tuple(x) for x in coords}) == 64


def test_hash_probe_limit_is_reported(gbf):
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 0, num_buckets=256, max_probe=4))
    d, c, T = H.frames(L, K, 1)[0]
    m.update(H.cuda(H.depth_m(d)), H.cuda(c), T)
    st = m.stats()
    assert st.status & L.FLAG_HASH_FULL
    assert 0 < st.allocated_blocks <= 256


def test_tiny_table_still_exact_when_it_fits(gbf):
    """Collision-heavy table (non-power-of-two slot count, long probe chains):
    the allocated set still equals the oracle's."""
    import oracle as O
    L = gbf
    K = H.intrinsics(L, 160, 120)
    cfg = H.small_config(L, 0, num_buckets=8191, max_probe=8191, num_blocks=6000)
    m = L.DenseMapping(K, cfg)
    om = O.OracleMap(O.config_from(cfg), O.intrinsics_from(K))
    for d, c, T in H.frames(L, K, 3, step=3):
        dm = H.depth_m(d)
        m.update(H.cuda(dm), H.cuda(c), T)
        om.fuse(dm, c, T)
    assert m.stats().status == 0
    g = H.sort_blocks(*m.export())
    o = H.sort_blocks(*om.export())
    for a, b in zip(g, o):
        assert np.array_equal(a, b)


def test_empty_and_invalid_frames(gbf):
    import torch
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 0))
    zero = torch.zeros((K.height, K.width), dtype=torch.float32, device="cuda")
    nan = torch.full((K.height, K.width), float("nan"), dtype=torch.float32, device="cuda")
    rgb = torch.zeros((K.height, K.width, 3), dtype=torch.uint8, device="cuda")
    for depth in (zero, nan):
        m.update(depth, rgb, np.eye(4))
        assert m.stats().allocated_blocks == 0 and m.stats().visible_blocks == 0
    vm = torch.full((K.height, K.width, 4), 7.0, device="cuda")
    m.raycast(vm, np.eye(4))
    # nothing visible: the raycast leaves the vertex map untouched (voxel_hashing.cpp:92-93)
    assert torch.all(vm == 7.0)


def test_lost_tracking_keeps_pose(gbf):
    import torch
    L = gbf
    K = H.intrinsics(L)
    s = L.System(K, H.small_config(L, 0))
    fr = H.frames(L, K, 1)
    s.set_pose(fr[0][2])
    s.process_images(H.cuda(fr[0][0]), H.cuda(fr[0][1]))
    blank = torch.zeros((K.height, K.width), dtype=torch.uint16, device="cuda")
    s.process_images(blank, H.cuda(fr[0][1]))
    st = s.stats()
    assert not st.track.success
    assert st.status & L.FLAG_TRACK_FAILED
    assert np.allclose(s.get_camera_pose(), fr[0][2])


def test_invalid_arguments_fail_cleanly(gbf):
    import torch
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 0))
    with pytest.raises(L.GbfError):
        L._lib.call("gbf_fuse", m.handle, None, K.width * 4, None, K.width * 3, None, 0, L._lib.mat16(np.eye(4)), None)
    vm = torch.zeros((K.height, K.width, 4), device="cuda")
    with pytest.raises(L.GbfError):
        L._lib.call("gbf_raycast", m.handle, L._lib.mat16(np.eye(4)), vm.data_ptr(), 16, None)
    # the session is still usable afterwards
    d, c, T = H.frames(L, K, 1)[0]
    m.update(H.cuda(H.depth_m(d)), H.cuda(c), T)
    assert m.stats().allocated_blocks > 0


def test_block_coordinates_out_of_range_are_flagged(gbf):
    """Blocks beyond the 21-bit key range (|block coordinate| >= 2^20: 84 km at
    1 cm voxels) are not allocated; the session raises COORD_RANGE and stays
    usable."""
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 0))
    d, c, T = H.frames(L, K, 1)[0]
    far = np.array(T, np.float64)
    far[0, 3] += 9.0e4  # 90 km along x
    m.update(H.cuda(H.depth_m(d)), H.cuda(c), far)
    st = m.stats()
    assert st.status & L.FLAG_COORD_RANGE
    assert st.allocated_blocks == 0
    m.update(H.cuda(H.depth_m(d)), H.cuda(c), T)  # back in range: fuses as usual
    assert m.stats().allocated_blocks > 0


def test_misaligned_images_are_rejected(gbf):
    """Images a kernel reads as float4 / float / u16 rows must start and step on
    their element size: a misaligned pitch or pointer is an argument error,
    not a device fault."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 0))
    buf = torch.zeros(K.height * K.width * 4 + 64, device="cuda")
    T = L._lib.mat16(np.eye(4))
    with pytest.raises(L.GbfError, match="aligned"):  # vertex-map pitch not a multiple of 16
        L._lib.call("gbf_raycast", m.handle, T, buf.data_ptr(), K.width * 16 + 4, None)
    with pytest.raises(L.GbfError, match="aligned"):  # vertex map starting 4 bytes off
        L._lib.call("gbf_raycast", m.handle, T, buf.data_ptr() + 4, K.width * 16, None)
    rgb = torch.zeros(K.height * K.width * 3, dtype=torch.uint8, device="cuda")
    with pytest.raises(L.GbfError, match="aligned"):  # depth pitch not a multiple of 4
        L._lib.call("gbf_fuse", m.handle, buf.data_ptr(), K.width * 4 + 2, rgb.data_ptr(), K.width * 3, None, 0,
                    T, None)
    # the session is still usable
    d, c, T2 = H.frames(L, K, 1)[0]
    m.update(H.cuda(H.depth_m(d)), H.cuda(c), T2)
    assert m.stats().allocated_blocks > 0


def test_positions_dropped_by_a_full_pool_allocate_after_pruning(gbf):
    """A block that found the pool full keeps its claimed table slot with no
    block behind it; that can only matter once room is made, and room is only
    made by deleting or pruning blocks, which rebuild the table from the
    allocated blocks alone.  So the next frame allocates positions the full
    pool had dropped."""
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 0, num_blocks=64))
    d, c, T = H.frames(L, K, 1)[0]
    depth, rgb = H.cuda(H.depth_m(d)), H.cuda(c)
    m.update(depth, rgb, T)
    first = {tuple(x) for x in m.export()[0]}
    assert len(first) == 64 and m.stats().status & L.FLAG_POOL_EXHAUSTED
    gone = np.array(sorted(first)[:32], np.int32)
    assert m.delete_blocks(gone) == 32
    assert m.stats().allocated_blocks == 32
    m.update(depth, rgb, T)
    second = {tuple(x) for x in m.export()[0]}
    assert len(second) == 64
    assert second - first, "only positions the pool had held before were allocated again"
    # every block pruned (radius 0 around the camera): the pool refills from the frame
    assert m.prune(center=T[:3, 3], radius=0.0) == 64
    assert m.stats().allocated_blocks == 0
    m.update(depth, rgb, T)
    assert m.stats().allocated_blocks == 64
