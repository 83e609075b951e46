"""End to end: System::process_images on the GPU against the FP32 oracle and
the ground-truth trajectory, and the batch path against single sessions."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _run_gpu(L, K, cfg, fr):
    s = L.System(K, cfg)
    s.set_pose(fr[0][2])
    poses = []
    for d, c, T in fr:
        s.process_images(H.cuda(d), H.cuda(c))
        poses.append(s.get_camera_pose())
    return s, poses


def test_system_matches_oracle_and_ground_truth(gbf):
    import oracle as O
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 0, bilateral=0)
    fr = H.frames(L, K, 12)
    s, gp = _run_gpu(L, K, cfg, fr)
    osys = O.OracleSystem(O.config_from(cfg), O.intrinsics_from(K))
    osys.set_pose(fr[0][2])
    op = []
    for d, c, T in fr:
        osys.process(d, c)
        op.append(osys.pose())
    gp, op = np.array(gp), np.array(op)
    truth = np.array([f[2] for f in fr])
    # drift of the GPU path against the oracle: <= 1 mm (the target bound)
    assert np.abs(gp[:, :3, 3] - op[:, :3, 3]).max() < 1e-3
    assert np.abs(gp[:, :3, :3] - op[:, :3, :3]).max() < 1e-3
    # and the tracker follows the synthetic trajectory
    assert np.abs(gp[:, :3, 3] - truth[:, :3, 3]).max() < 0.02
    st = s.stats()
    assert st.status == 0 and st.frame_index == len(fr)
    gc = H.sort_blocks(s.export()[0])[0]
    oc = H.sort_blocks(osys.map_export()[0])[0]
    a = {tuple(x) for x in gc}
    b = {tuple(x) for x in oc}
    assert len(a & b) / len(a | b) > 0.99


def test_batch_session_isolation(gbf):
    """A session gives the same result alone and batched with others of other
    resolutions / voxel sizes / voxel layouts (bit-identical pose and map)."""
    import torch
    L = gbf
    KA = H.intrinsics(L, 320, 240)
    KB = H.intrinsics(L, 160, 120)
    KC = H.intrinsics(L, 256, 192)
    cfgA = H.small_config(L, 0)
    cfgB = H.small_config(L, 1, voxel_size=0.016, truncation=0.048)
    cfgC = H.small_config(L, 2, voxel_size=0.008, truncation=0.03)
    frA = H.frames(L, KA, 5, seed=3)
    frB = H.frames(L, KB, 5, seed=9)
    frC = H.frames(L, KC, 5, seed=11)

    def run_alone(K, cfg, fr):
        s = L.System(K, cfg)
        s.set_pose(fr[0][2])
        for d, c, T in fr:
            s.process_images(H.cuda(d), H.cuda(c))
        return s.get_camera_pose(), s.export()

    pa, ma = run_alone(KA, cfgA, frA)
    pc, mc = run_alone(KC, cfgC, frC)

    for use_graph, groups in ((False, 1), (True, 1), (False, 2), (True, 3)):
        a = L.System(KA, cfgA)
        b = L.System(KB, cfgB)
        b2 = L.System(KB, cfgB)
        cc = L.System(KC, cfgC)
        a.set_pose(frA[0][2])
        b.set_pose(frB[0][2])
        b2.set_pose(frB[0][2])
        cc.set_pose(frC[0][2])
        batch = L.FusionBatch(5)
        batch.set(0, b)
        batch.set(1, cc)
        batch.set(2, a)
        batch.set(3, b2)
        batch.set_groups(groups)
        for i in range(5):
            for sess, (d, c, T) in ((a, frA[i]), (b, frB[i]), (b2, frB[i]), (cc, frC[i])):
                sess.stage(H.cuda(d), H.cuda(c))
            batch.process([True, True, True, True, True], use_graph=use_graph)
            torch.cuda.synchronize()
        assert np.array_equal(a.get_camera_pose(), pa)
        assert np.array_equal(cc.get_camera_pose(), pc)
        batch.flush()  # the staggered group's last frame is fused here
        for alone_map, sess in ((ma, a), (mc, cc)):
            mb = sess.export()
            for x, y in zip(alone_map, mb):
                xs = H.sort_blocks(alone_map[0], x)[1]
                ys = H.sort_blocks(mb[0], y)[1]
                assert np.array_equal(xs, ys)
        # the two identical B sessions agree with each other
        assert np.array_equal(b.get_camera_pose(), b2.get_camera_pose())
        batch.close()




def test_step_launch_of_a_large_batch_matches_sessions_alone(gbf):
    """A launch of 32 or more sessions takes each session's partial-record sum
    and Gauss-Newton step in a launch of its own (gn_step_kernel); a session
    alone takes them in the reduction's last CTA.  32 sessions in one launch
    give every session, frame by frame, the poses it has alone, bit for bit."""
    import torch
    L = gbf
    K = H.intrinsics(L, 160, 120)
    n, nf = 32, 4
    fr = {seed: H.frames(L, K, nf, seed=seed) for seed in (3, 9, 11, 17)}
    seeds = [(3, 9, 11, 17)[i % 4] for i in range(n)]
    cfgs = [H.small_config(L, i % 3, num_blocks=1 << 13, num_buckets=1 << 15) for i in range(n)]

    alone = []
    for i in range(n):
        s = L.System(K, cfgs[i])
        s.set_pose(fr[seeds[i]][0][2])
        poses = []
        for d, c, _ in fr[seeds[i]]:
            s.process_images(H.cuda(d), H.cuda(c))
            poses.append(s.get_camera_pose())
        alone.append(poses)
        s.close()

    sess = [L.System(K, cfgs[i]) for i in range(n)]
    batch = L.FusionBatch(n)
    for i, s in enumerate(sess):
        s.set_pose(fr[seeds[i]][0][2])
        batch.set(i, s)
    batch.set_groups(1)
    for k in range(nf):
        for i, s in enumerate(sess):
            d, c, _ = fr[seeds[i]][k]
            s.stage(H.cuda(d), H.cuda(c))
        batch.process([True] * n, use_graph=True)
        torch.cuda.synchronize()
        for i, s in enumerate(sess):
            assert np.array_equal(s.get_camera_pose(), alone[i][k]), (i, k)
    batch.close()
    for s in sess:
        s.close()


def test_pitched_staging_matches_dense_staging(gbf):
    """Frames staged from pitched rows (a camera buffer wider than the image,
    pinned host and device memory) give the same poses and map as the same
    frames staged from dense rows: dense rows go as one contiguous copy, pitched
    ones row by row."""
    import ctypes as C
    import torch
    from libfusion_gb300 import call
    L = gbf
    K = H.intrinsics(L, 320, 240)
    W, Hh = K.width, K.height
    fr = H.frames(L, K, 4, seed=5)

    def run(pitched, host):
        s = L.System(K, H.small_config(L, 2))
        s.set_pose(fr[0][2])
        poses = []
        for d, c, _ in fr:
            if pitched:
                dp = torch.zeros((Hh, W + 24), dtype=torch.uint16)
                cp = torch.zeros((Hh, W * 3 + 40), dtype=torch.uint8)
                dp[:, :W] = torch.from_numpy(d)
                cp[:, :W * 3] = torch.from_numpy(np.ascontiguousarray(c).reshape(Hh, W * 3))
            else:
                dp, cp = torch.from_numpy(np.ascontiguousarray(d)), torch.from_numpy(np.ascontiguousarray(c))
            dp = dp.pin_memory() if host else dp.cuda()
            cp = cp.pin_memory() if host else cp.cuda()
            call("gbf_session_stage", s._h, dp.data_ptr(), dp.stride(0) * 2, cp.data_ptr(),
                 cp.stride(0) if pitched else W * 3, C.c_void_p(0))
            s.process_staged()
            poses.append(s.get_camera_pose())
        torch.cuda.synchronize()
        out = poses, s.export()
        s.close()
        return out

    for host in (True, False):
        pd, md = run(False, host)
        pp, mp = run(True, host)
        assert all(np.array_equal(a, b) for a, b in zip(pd, pp))
        for x, y in zip(md, mp):  # blocks in coordinate order (ids follow insertion order)
            assert np.array_equal(H.sort_blocks(md[0], x)[1], H.sort_blocks(mp[0], y)[1])

def test_batch_staging_pipeline_matches_session_staging(gbf):
    """Frames staged into the batch's double-buffered inputs on a copy stream,
    one tick ahead of the compute, and results read one tick behind give the
    same poses and maps as staging into each session before every tick."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    fr = [H.frames(L, K, 6, seed=s) for s in (4, 5)]
    host = [[(torch.from_numpy(d).pin_memory(), torch.from_numpy(c).pin_memory()) for d, c, _ in f] for f in fr]

    def run(pipelined):
        ss = [L.System(K, cfg) for _ in range(2)]
        for s, f in zip(ss, fr):
            s.set_pose(f[0][2])
        b = L.FusionBatch(2)
        for i, s in enumerate(ss):
            b.set(i, s)
        copy = torch.cuda.Stream()
        seen = []
        for k in range(6):
            for i, s in enumerate(ss):
                if pipelined:
                    b.stage(i, host[i][k][0], host[i][k][1], stream=copy)
                else:
                    s.stage(H.cuda(fr[i][k][0]), H.cuda(fr[i][k][1]))
            b.process([True, True])
            if pipelined and k > 0:
                seen.append(b.results(back=1))
        last = b.results(back=0)
        b.flush()
        torch.cuda.synchronize()
        poses = [s.get_camera_pose() for s in ss]
        maps = [s.export() for s in ss]
        b.close()
        return poses, maps, seen, last

    p0, m0, _, last0 = run(False)
    p1, m1, seen, last1 = run(True)
    for a, b in zip(p0, p1):
        assert np.array_equal(a, b)
    for a, b in zip(m0, m1):
        for x, y in zip(H.sort_blocks(*a), H.sort_blocks(*b)):
            assert np.array_equal(x, y)
    # the result records carry the poses, one record per tick, in order
    for i in range(2):
        assert np.array_equal(last1[0][i], p1[i])
        assert last1[3][i] == 6
    assert [int(r[3][0]) for r in seen] == [1, 2, 3, 4, 5]


def test_staggered_groups_same_results(gbf):
    """Odd groups half a frame out of phase: every tick's poses and, after a
    flush, every map equal those of the unstaggered batch; changing the layout
    mid-run (groups, stagger, slot assignment) flushes what is owed first."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    n = 4
    fr = [H.frames(L, K, 6, seed=20 + i) for i in range(n)]

    def run(stagger, switch_at=None):
        ss = [L.System(K, cfg) for _ in range(n)]
        for s, f in zip(ss, fr):
            s.set_pose(f[0][2])
        b = L.FusionBatch(n)
        for i, s in enumerate(ss):
            b.set(i, s)
        b.set_groups(2)
        b.set_stagger(stagger)
        poses = []
        for k in range(6):
            if switch_at is not None and k == switch_at:
                b.set_stagger(not stagger)
            for i, s in enumerate(ss):
                s.stage(H.cuda(fr[i][k][0]), H.cuda(fr[i][k][1]))
            b.process([True] * n)
            poses.append(b.results(back=0)[0])
        b.flush()
        torch.cuda.synchronize()
        maps = [s.export() for s in ss]
        b.close()
        return poses, maps

    p0, m0 = run(False)
    for args in ((True,), (True, 3)):
        p1, m1 = run(*args)
        for x, y in zip(p0, p1):
            assert np.array_equal(x, y)
        for a, b in zip(m0, m1):
            for x, y in zip(H.sort_blocks(*a), H.sort_blocks(*b)):
                assert np.array_equal(x, y)


def test_batch_churn_keeps_graph_and_results(gbf):
    """Serving churn: a session evicted and a new one of the same shape admitted
    into its slot between graph ticks.  The newcomer's poses and map equal the
    same frames processed alone, and the neighbours are undisturbed."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    fr = [H.frames(L, K, 6, seed=40 + i) for i in range(4)]

    def alone(f, frames):
        s = L.System(K, cfg)
        s.set_pose(f[frames[0]][2])
        for k in frames:
            s.process_images(H.cuda(f[k][0]), H.cuda(f[k][1]))
        torch.cuda.synchronize()
        return s.get_camera_pose(), s.export()

    ss = [L.System(K, cfg) for _ in range(3)]
    for s, f in zip(ss, fr):
        s.set_pose(f[0][2])
    b = L.FusionBatch(3)
    for i, s in enumerate(ss):
        b.set(i, s)
    for k in range(6):
        if k == 3:  # evict slot 1, admit a fresh session on another sequence
            newcomer = L.System(K, cfg)
            newcomer.set_pose(fr[3][3][2])
            b.set(1, newcomer)
            ss[1] = newcomer
        for i, s in enumerate(ss):
            f = fr[3] if (i == 1 and k >= 3) else fr[i]
            s.stage(H.cuda(f[k][0]), H.cuda(f[k][1]))
        b.process([True, True, True], use_graph=True)
    b.flush()
    torch.cuda.synchronize()
    for s, (pose, m) in ((ss[0], alone(fr[0], range(6))), (ss[1], alone(fr[3], range(3, 6))),
                         (ss[2], alone(fr[2], range(6)))):
        assert np.array_equal(s.get_camera_pose(), pose)
        for x, y in zip(H.sort_blocks(*s.export()), H.sort_blocks(*m)):
            assert np.array_equal(x, y)
    b.close()


def test_reserved_batch_admits_smaller_sessions_without_recapture(gbf):
    """A batch reserved for three slots of the largest configuration it serves
    admits and evicts sessions of a smaller block pool, and leaves a slot empty,
    without capturing its tick again: two graphs (one per tick parity) for the
    whole run.  Every session's poses and map equal the same frames processed
    alone.  The same churn in a batch with no reservation re-captures."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    big = H.small_config(L, 1)
    small = H.small_config(L, 1, num_blocks=1 << 14, num_buckets=1 << 16)
    fr = [H.frames(L, K, 6, seed=70 + i) for i in range(4)]
    # (slot, config, sequence, first tick, last tick + 1)
    plan = [(0, small, 0, 0, 6), (1, big, 1, 0, 3), (2, small, 2, 2, 6), (1, small, 3, 3, 6)]

    def alone(cfg, f, frames):
        s = L.System(K, cfg)
        s.set_pose(f[frames[0]][2])
        for k in frames:
            s.process_images(H.cuda(f[k][0]), H.cuda(f[k][1]))
        torch.cuda.synchronize()
        return s.get_camera_pose(), s.export()

    def run(reserve):
        b = L.FusionBatch(3)
        if reserve:
            b.reserve(K, big, 3)
        slots, done = [None] * 3, []
        for k in range(6):
            for j, (slot, cfg, seq, k0, k1) in enumerate(plan):
                if k == k1 and slots[slot] is not None and slots[slot][0] == j:
                    b.flush()
                    torch.cuda.synchronize()
                    done.append((j, slots[slot][1].get_camera_pose(), slots[slot][1].export()))
                    b.set(slot, None)
                    slots[slot] = None
            for j, (slot, cfg, seq, k0, k1) in enumerate(plan):
                if k == k0:
                    s = L.System(K, cfg)
                    s.set_pose(fr[seq][k][2])
                    b.set(slot, s)
                    slots[slot] = (j, s)
            active = [x is not None for x in slots]
            for slot, x in enumerate(slots):
                if x is not None:
                    f = fr[plan[x[0]][2]][k]
                    x[1].stage(H.cuda(f[0]), H.cuda(f[1]))
            b.process(active, use_graph=True)
            if k == 1:
                first = b.captures()
        b.flush()
        torch.cuda.synchronize()
        for x in slots:
            if x is not None:
                done.append((x[0], x[1].get_camera_pose(), x[1].export()))
        n = b.captures()
        b.close()
        return sorted(done, key=lambda d: d[0]), first, n

    got, first, n = run(True)
    assert first == 2 and n == 2, (first, n)
    assert [d[0] for d in got] == list(range(len(plan)))
    for (j, pose, m), (slot, cfg, seq, k0, k1) in zip(got, plan):
        want_pose, want_map = alone(cfg, fr[seq], range(k0, k1))
        assert np.array_equal(pose, want_pose), j
        for x, y in zip(H.sort_blocks(*m), H.sort_blocks(*want_map)):
            assert np.array_equal(x, y), j
    got2, _, n2 = run(False)
    assert n2 > 2
    for a, c in zip(got, got2):
        assert np.array_equal(a[1], c[1])


def test_autotune_explores_settles_and_keeps_results(gbf):
    """The online tuner switches groups, stagger and raycast tile while the batch
    serves: every tick's poses and the final maps equal those of a batch with a
    fixed launch shape; it settles on the candidate with the fastest median, and
    a second batch of the same shape settles from the process-wide table."""
    import torch
    L = gbf
    L.autotune_forget()
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    n, ticks = 4, 48
    fr = [H.frames(L, K, ticks, seed=60 + i) for i in range(n)]

    def run(tune):
        ss = [L.System(K, cfg) for _ in range(n)]
        for s, f in zip(ss, fr):
            s.set_pose(f[0][2])
        b = L.FusionBatch(n)
        for i, s in enumerate(ss):
            b.set(i, s)
        if tune:
            b.autotune(True, 2)
        else:
            b.set_groups(2)
        poses = []
        for k in range(ticks):
            for i, s in enumerate(ss):
                s.stage(H.cuda(fr[i][k][0]), H.cuda(fr[i][k][1]))
            b.process([True] * n)
            poses.append(b.results(back=0)[0])
        b.flush()
        torch.cuda.synchronize()
        t = b.tuning()
        maps = [s.export() for s in ss]
        b.close()
        return poses, maps, t

    p0, m0, t0 = run(False)
    assert t0["state"] == "off"
    p1, m1, t1 = run(True)
    for x, y in zip(p0, p1):
        assert np.array_equal(x, y)
    for a, c in zip(m0, m1):
        for x, y in zip(H.sort_blocks(*a), H.sort_blocks(*c)):
            assert np.array_equal(x, y)
    print("tuning:", t1)
    assert t1["state"] == "settled" and not t1["from_table"]
    tried = t1["tried"]
    # groups 1..4 x stagger at the 8-wide tile (7), then tiles 4, 16 and 32 at the best
    assert len(tried) == 10
    assert {(c["groups"], c["stagger"]) for c in tried[:7]} == {(1, 0), (2, 0), (2, 1), (3, 0), (3, 1), (4, 0), (4, 1)}
    assert [c["ray_tile_w"] for c in tried[7:]] == [4, 16, 32]
    best = min(tried, key=lambda c: c["median_ms"])
    ch = t1["chosen"]
    assert (ch["groups"], ch["stagger"], ch["ray_tile_w"]) == (best["groups"], best["stagger"], best["ray_tile_w"])
    assert all(c["median_ms"] > 0 for c in tried)

    # a batch of the same shape starts from the table
    ss = [L.System(K, cfg) for _ in range(n)]
    b = L.FusionBatch(n)
    for i, s in enumerate(ss):
        s.set_pose(fr[i][0][2])
        b.set(i, s)
    b.autotune(True, 2)
    for i, s in enumerate(ss):
        s.stage(H.cuda(fr[i][0][0]), H.cuda(fr[i][0][1]))
    b.process([True] * n)
    t2 = b.tuning()
    assert t2["state"] == "settled" and t2["from_table"]
    assert t2["chosen"]["groups"] == ch["groups"] and t2["chosen"]["ray_tile_w"] == ch["ray_tile_w"]
    b.close()
    L.autotune_forget()


@pytest.mark.parametrize("tile_w", [4, 16, 32])
def test_ray_tile_same_raycast(gbf, tile_w):
    """A batch's raycast tile width changes the launch, not the vertex maps."""
    import torch
    L = gbf
    K = H.intrinsics(L, 328, 248)  # ragged: no tile shape divides it
    cfg = H.small_config(L, 1)
    fr = H.frames(L, K, 3, seed=70)
    out = []
    for tw in (8, tile_w):
        s = L.System(K, cfg)
        s.set_pose(fr[0][2])
        b = L.FusionBatch(1)
        b.set(0, s)
        b.set_ray_tile(tw)
        for d, c, _ in fr:
            s.stage(H.cuda(d), H.cuda(c))
            b.process([True])
        b.flush()
        torch.cuda.synchronize()
        vm = s.get_image(1, 0, 0)  # the reference set's level-0 vertex map: the last raycast
        torch.cuda.synchronize()
        out.append((s.get_camera_pose(), s.export(), vm.cpu().numpy()))
        b.close()
    assert np.array_equal(out[0][0], out[1][0])
    for x, y in zip(H.sort_blocks(*out[0][1]), H.sort_blocks(*out[1][1])):
        assert np.array_equal(x, y)
    assert np.array_equal(np.nan_to_num(out[0][2], nan=7.0), np.nan_to_num(out[1][2], nan=7.0))


def test_inactive_slot_skips_its_ticks(gbf):
    """A slot marked inactive for some ticks is left as it was: its session
    ends equal to the same session fed only its active frames, and its
    neighbour is undisturbed."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    fa = H.frames(L, K, 5, seed=50)
    fb = H.frames(L, K, 5, seed=51)
    skip = {1, 2}  # ticks on which slot 1 is inactive

    def alone(fr, ticks):
        s = L.System(K, cfg)
        s.set_pose(fr[0][2])
        for k in ticks:
            s.process_images(H.cuda(fr[k][0]), H.cuda(fr[k][1]))
        torch.cuda.synchronize()
        return s.get_camera_pose(), s.export()

    a, b = L.System(K, cfg), L.System(K, cfg)
    a.set_pose(fa[0][2])
    b.set_pose(fb[0][2])
    batch = L.FusionBatch(2)
    batch.set(0, a)
    batch.set(1, b)
    for k in range(5):
        a.stage(H.cuda(fa[k][0]), H.cuda(fa[k][1]))
        if k not in skip:
            b.stage(H.cuda(fb[k][0]), H.cuda(fb[k][1]))
        batch.process([True, k not in skip])
    batch.flush()
    torch.cuda.synchronize()
    for sess, (pose, m) in ((a, alone(fa, range(5))), (b, alone(fb, [k for k in range(5) if k not in skip]))):
        assert np.array_equal(sess.get_camera_pose(), pose)
        for x, y in zip(H.sort_blocks(*sess.export()), H.sort_blocks(*m)):
            assert np.array_equal(x, y)
    assert b.stats().frame_index == 3 and a.stats().frame_index == 5
    batch.close()


def test_batch_calls_from_several_threads(gbf):
    """The batch is internally synchronised: camera threads stage their own
    session's frames from pinned host memory, a monitor thread reads the tuner
    and launch counts, and the main thread runs the ticks and reads results;
    every session ends bit-identical to the same frames processed alone."""
    import threading

    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 1)
    n, ticks = 4, 6
    fr = [H.frames(L, K, ticks, seed=80 + i) for i in range(n)]
    host = [[(torch.from_numpy(d).pin_memory(), torch.from_numpy(c).pin_memory()) for d, c, _ in f] for f in fr]
    ss = [L.System(K, cfg) for _ in range(n)]
    for s, f in zip(ss, fr):
        s.set_pose(f[0][2])
    batch = L.FusionBatch(n)
    for i, s in enumerate(ss):
        batch.set(i, s)
    batch.autotune(True, 2)
    stop = threading.Event()
    seen = []

    def monitor():
        while not stop.is_set():
            seen.append((batch.tuning()["state"], batch.kernels_per_tick()))

    mon = threading.Thread(target=monitor)
    mon.start()
    streams = [torch.cuda.Stream() for _ in range(n)]
    try:
        for k in range(ticks):
            def stage(i):
                batch.stage(i, host[i][k][0], host[i][k][1], stream=streams[i])
            cams = [threading.Thread(target=stage, args=(i,)) for i in range(n)]
            for t in cams:
                t.start()
            for t in cams:
                t.join()
            batch.process([True] * n)
            batch.results(back=0)
    finally:
        stop.set()
        mon.join()
    batch.flush()
    torch.cuda.synchronize()
    assert seen
    for i, s in enumerate(ss):
        alone = L.System(K, cfg)
        alone.set_pose(fr[i][0][2])
        for d, c, _ in fr[i]:
            alone.process_images(H.cuda(d), H.cuda(c))
        torch.cuda.synchronize()
        assert np.array_equal(s.get_camera_pose(), alone.get_camera_pose())
        for x, y in zip(H.sort_blocks(*s.export()), H.sort_blocks(*alone.export())):
            assert np.array_equal(x, y)
    batch.close()


def test_motion_prior_matches_oracle(gbf):
    """With the constant-velocity prior (motion_prior = 1) each frame's
    Gauss-Newton starts from the motion the last frame tracked; the GPU loop
    follows the FP32 oracle's within the same bound as without it, on frames
    two steps apart (faster motion)."""
    import oracle as O
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 0, bilateral=0, motion_prior=1)
    fr = H.frames(L, K, 10, step=2)
    s, gp = _run_gpu(L, K, cfg, fr)
    osys = O.OracleSystem(O.config_from(cfg), O.intrinsics_from(K))
    osys.set_pose(fr[0][2])
    ok = []
    for d, c, T in fr:
        osys.process(d, c)
        ok.append(osys.last_result().success)
    gp = np.array(gp)
    assert np.abs(gp[-1, :3, 3] - osys.pose()[:3, 3]).max() < 1e-3
    assert bool(s.stats().track.success) == bool(ok[-1])
    truth = np.array([f[2] for f in fr])
    assert np.abs(gp[:, :3, 3] - truth[:, :3, 3]).max() < 0.02


@pytest.mark.parametrize("collect", [False, True])
def test_server_results_alone_and_in_the_mix(gbf, collect):
    """The continuous-batching server (libfusion_gb300/serving.py) on the GPU:
    three requests of two voxel sizes through a two-slot batch whose memory
    budget holds two session arenas.  The third request waits for a slot,
    takes the memory of an evicted session, and every session's poses, frame
    by frame, equal those of the same frames run alone on the plain path, bit
    for bit, whatever else shared its ticks.  With collection, every third
    fused frame of a session prunes its map around the tracked camera between
    ticks (gbf_map_prune_async on the server's stream); the plain path prunes
    synchronously after the same frames."""
    import torch
    from libfusion_gb300.serving import ArenaCache, Request, Server
    L = gbf
    K = H.intrinsics(L)
    cfgs = {8: H.small_config(L, 2, voxel_size=0.008, truncation=0.024),
            10: H.small_config(L, 2, voxel_size=0.01)}
    nbytes = {v: L.session_bytes(c, K) for v, c in cfgs.items()}
    spec = [(0, 0.0, 8, 12, 3), (1, 0.0, 10, 9, 4), (2, 0.02, 8, 10, 5)]  # sid, arrival, voxel mm, frames, seed
    frames = {}
    for sid, _, _, n, seed in spec:
        sc = L.SynthScene(seed=seed)
        d = torch.empty((n, K.height, K.width), dtype=torch.uint16, device="cuda")
        c = torch.empty((n, K.height, K.width, 3), dtype=torch.uint8, device="cuda")
        for k in range(n):
            sc.render_into(K, k, d[k].data_ptr(), c[k].data_ptr())
        frames[sid] = (d, c, sc.pose(0))
        sc.close()
    torch.cuda.synchronize()
    batch = L.FusionBatch(2)
    batch.reserve(K, cfgs[8], 2)
    batch.set_groups(1)
    cache = ArenaCache(nbytes[8] + nbytes[10], make=lambda key: L.System(K, cfgs[key[0]]),
                       destroy=lambda s: s.close(), reset=lambda s: s.reset())
    every, radius = 3, 1.2

    def prune(s, pose, stream):
        s.prune_async(center=np.asarray(pose)[:3, 3], radius=radius, drop_unobserved=True, stream=stream)

    srv = Server(batch, 2, cache, record_poses=True, collect=prune if collect else None, collect_every=every)
    for sid, t, v, n, _ in spec:
        d, c, T0 = frames[sid]
        srv.submit(Request(sid=sid, arrival=t, frames=n, key=(v,), nbytes=nbytes[v], pose0=T0, fps=200.0,
                           source=lambda k, d=d, c=c: (d[k].data_ptr(), c[k].data_ptr())))
    srv.run(10.0)
    rep = srv.report()
    assert rep["completed"] == 3 and rep["frames"] == sum(n for _, _, _, n, _ in spec)
    assert rep["deferred_by_slots"] >= 1 and rep["concurrency_peak"] == 2
    assert rep["memory"]["peak_bytes"] <= nbytes[8] + nbytes[10]
    assert rep["tracking_failed_frames"] == 0
    assert rep["collections"] == (sum((n - 1) // every for _, _, _, n, _ in spec) if collect else 0)
    batch.close()
    cache.close()
    pruned = 0
    for sid, _, v, n, _ in spec:
        d, c, T0 = frames[sid]
        s = L.System(K, cfgs[v])
        s.set_pose(T0)
        for k in range(n):
            s.process_images(d[k], c[k])
            pose = s.get_camera_pose()
            assert np.array_equal(pose, srv.poses[(sid, k)]), (sid, k)
            if collect and (k + 1) % every == 0 and k + 1 < n:
                pruned += s.prune(center=pose[:3, 3], radius=radius, drop_unobserved=True)
        s.close()
    assert pruned > 0 or not collect


def test_prune_between_graph_ticks_matches_session_alone(gbf):
    """Serving loop garbage collection: one session of a two-slot batch prunes
    its map (radius around its camera, and unobserved blocks) on the batch's
    stream between two graph ticks, with no host synchronisation.  Its poses and
    map equal the same frames processed alone with a synchronous prune at the
    same frame; the other session is undisturbed."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    cfg = H.small_config(L, 2)
    n_fr, at = 6, 3
    fr = [H.frames(L, K, n_fr, seed=90 + i) for i in range(2)]
    radius = 1.2

    def alone(i, prune):
        s = L.System(K, cfg)
        s.set_pose(fr[i][0][2])
        for k, (d, c, T) in enumerate(fr[i]):
            if prune and k == at:
                n = s.prune(center=s.get_camera_pose()[:3, 3], radius=radius, drop_unobserved=True)
                assert n > 0
            s.process_images(H.cuda(d), H.cuda(c))
        torch.cuda.synchronize()
        return s.get_camera_pose(), s.export()

    ss = [L.System(K, cfg) for _ in range(2)]
    for s, f in zip(ss, fr):
        s.set_pose(f[0][2])
    b = L.FusionBatch(2)
    for i, s in enumerate(ss):
        b.set(i, s)
    stream = torch.cuda.current_stream()
    for k in range(n_fr):
        if k == at:
            b.flush()
            torch.cuda.synchronize()
            cam = ss[0].get_camera_pose()[:3, 3]
            n_before = ss[0].stats().allocated_blocks
            ss[0].prune_async(center=cam, radius=radius, drop_unobserved=True, stream=stream)
        for i, s in enumerate(ss):
            s.stage(H.cuda(fr[i][k][0]), H.cuda(fr[i][k][1]))
        b.process([True, True], use_graph=True, stream=stream)
    b.flush()
    torch.cuda.synchronize()
    for i, s in enumerate(ss):
        pose, m = alone(i, prune=(i == 0))
        assert np.array_equal(s.get_camera_pose(), pose), i
        for x, y in zip(H.sort_blocks(*s.export()), H.sort_blocks(*m)):
            assert np.array_equal(x, y), i
    b.close()
    assert n_before > 0
