"""Session snapshot and restore (evict a serving session to host memory and
resume it): a restored session continues bit for bit as the original would
have -- poses frame by frame and the final map -- in every voxel layout, from
host or device memory, in a fresh session or in a batch slot; snapshots of
another configuration or a damaged header are refused."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _run(L, K, cfg, fr, frames, s=None):
    import torch
    if s is None:
        s = L.System(K, cfg)
        s.set_pose(fr[frames[0]][2])
    poses = []
    for k in frames:
        s.process_images(H.cuda(fr[k][0]), H.cuda(fr[k][1]))
        poses.append(s.get_camera_pose())
    torch.cuda.synchronize()
    return s, poses


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_restored_session_continues_bit_for_bit(gbf, layout):
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, layout, motion_prior=1)
    n, cut = 8, 4
    fr = H.frames(L, K, n, step=2)
    whole, want = _run(L, K, cfg, fr, range(n))
    a, first = _run(L, K, cfg, fr, range(cut))
    assert all(np.array_equal(x, y) for x, y in zip(first, want[:cut]))
    snap = a.snapshot()
    assert len(snap) == a.snapshot_bytes()
    stats_a = a.stats()
    a.close()
    b = L.System(K, cfg)
    b.restore(snap)
    st = b.stats()
    assert st.frame_index == stats_a.frame_index and st.allocated_blocks == stats_a.allocated_blocks
    assert np.array_equal(b.get_camera_pose(), first[-1])
    b, rest = _run(L, K, cfg, fr, range(cut, n), s=b)
    for k, (x, y) in enumerate(zip(rest, want[cut:])):
        assert np.array_equal(x, y), cut + k
    for x, y in zip(H.sort_blocks(*b.export()), H.sort_blocks(*whole.export())):
        assert np.array_equal(x, y)
    assert b.stats().status == whole.stats().status


def test_snapshot_in_device_memory_and_into_a_batch_slot(gbf):
    """A session of a two-slot batch is evicted to a device buffer half way and
    resumed later into the other slot of the same batch (its first slot taken by
    another session meanwhile): every frame's pose equals the same frames run
    alone."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 2)
    n, cut = 8, 3
    fr = [H.frames(L, K, n, seed=110 + i) for i in range(3)]
    _, want0 = _run(L, K, cfg, fr[0], range(n))
    _, want2 = _run(L, K, cfg, fr[2], range(n))
    s0, s1 = L.System(K, cfg), L.System(K, cfg)
    s0.set_pose(fr[0][0][2])
    s1.set_pose(fr[2][0][2])
    b = L.FusionBatch(2)
    b.set(0, s0)
    got0, got2 = [], []
    buf = torch.empty(1 << 30, dtype=torch.uint8, device="cuda")
    snap = None
    for k in range(n):
        if k == cut:  # evict session 0 to device memory, slot 0 to the other camera
            b.flush()
            torch.cuda.synchronize()
            snap = s0.snapshot(out=buf)
            b.set(0, s1)
            s0.close()
        if k == cut + 2:  # resume session 0 in slot 1 from its snapshot, two frames late
            r = L.System(K, cfg)
            r.restore(snap)
            b.set(1, r)
            s0 = r
        active = [True, k >= cut + 2]
        if k < cut:
            s0.stage(H.cuda(fr[0][k][0]), H.cuda(fr[0][k][1]))
            active = [True, False]
        else:
            j = k - cut  # camera 2's frames, from its first
            s1.stage(H.cuda(fr[2][j][0]), H.cuda(fr[2][j][1]))
            if k >= cut + 2:
                m = k - 2  # camera 0 resumes where it stopped
                s0.stage(H.cuda(fr[0][m][0]), H.cuda(fr[0][m][1]))
        b.process(active, use_graph=True)
        poses = b.results(back=0)[0]
        if k < cut:
            got0.append(poses[0])
        else:
            got2.append(poses[0])
            if k >= cut + 2:
                got0.append(poses[1])
    b.flush()
    torch.cuda.synchronize()
    b.close()
    assert len(got0) == n - 2 and len(got2) == n - cut
    for k, (x, y) in enumerate(zip(got0, want0)):
        assert np.array_equal(x, y), k
    for k, (x, y) in enumerate(zip(got2, want2)):
        assert np.array_equal(x, y), k


def test_restore_refuses_other_configurations_and_damaged_snapshots(gbf):
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    fr = H.frames(L, K, 2)
    a, _ = _run(L, K, cfg, fr, range(2))
    snap = a.snapshot()
    other = L.System(K, H.small_config(L, 1, num_blocks=1 << 14))
    with pytest.raises(L.GbfError) as e:
        other.restore(snap)
    assert e.value.status == 1
    small = L.System(H.intrinsics(L, 160, 120), cfg)
    with pytest.raises(L.GbfError):
        small.restore(snap)
    bad = snap.copy()
    bad[0] ^= 0xFF
    b = L.System(K, cfg)
    with pytest.raises(L.GbfError):
        b.restore(bad)
    with pytest.raises(L.GbfError):
        b.restore(snap[: len(snap) // 2])
    with pytest.raises(L.GbfError) as e:
        a.snapshot(out=np.empty(64, np.uint8))
    assert e.value.status == 4  # GBF_ERR_CAPACITY
    b.restore(snap)  # the intact snapshot still restores
    assert b.stats().allocated_blocks == a.stats().allocated_blocks


def test_server_parks_a_paused_session_and_resumes_it_bit_for_bit(gbf):
    """The server with one slot and memory for one arena: camera 0 pauses after
    its fourth frame, its session is snapshotted to host memory and its arena
    goes to camera 1, which arrives during the pause and runs to its end in the
    same arena; camera 0 then resumes in that arena again.  Every frame's pose
    of both cameras equals the same frames run alone."""
    import torch
    from libfusion_gb300.serving import ArenaCache, Request, Server
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 2)
    nbytes = L.session_bytes(cfg, K)
    spec = [(0, 0.0, 8, 21, {3: 0.4}), (1, 0.08, 5, 22, None)]  # sid, arrival, frames, seed, pauses
    frames = {}
    for sid, _, n, seed, _ in spec:
        sc = L.SynthScene(seed=seed)
        d = torch.empty((n, K.height, K.width), dtype=torch.uint16, device="cuda")
        c = torch.empty((n, K.height, K.width, 3), dtype=torch.uint8, device="cuda")
        for k in range(n):
            sc.render_into(K, k, d[k].data_ptr(), c[k].data_ptr())
        frames[sid] = (d, c, sc.pose(0))
        sc.close()
    torch.cuda.synchronize()
    batch = L.FusionBatch(1)
    cache = ArenaCache(nbytes, make=lambda key: L.System(K, cfg), destroy=lambda s: s.close(),
                       reset=lambda s: s.reset())
    srv = Server(batch, 1, cache, record_poses=True, park_after=0.05, snapshot=lambda s: s.snapshot(),
                 restore=lambda s, snap: s.restore(snap))
    for sid, t, n, _, pauses in spec:
        d, c, T0 = frames[sid]
        srv.submit(Request(sid=sid, arrival=t, frames=n, key=("a",), nbytes=nbytes, pose0=T0, fps=100.0,
                           pauses=pauses, source=lambda k, d=d, c=c: (d[k].data_ptr(), c[k].data_ptr())))
    srv.run(5.0)
    rep = srv.report()
    assert rep["completed"] == 2 and rep["frames"] == 13
    assert rep["parking"]["parked"] == 1 and rep["parking"]["resumed"] == 1
    assert rep["memory"]["arenas_created"] == 1 and rep["tracking_failed_frames"] == 0
    batch.close()
    cache.close()
    for sid, _, n, _, _ in spec:
        d, c, T0 = frames[sid]
        s = L.System(K, cfg)
        s.set_pose(T0)
        for k in range(n):
            s.process_images(d[k], c[k])
            assert np.array_equal(s.get_camera_pose(), srv.poses[(sid, k)]), (sid, k)
        s.close()
