"""Map dump in the reference's raw layout (MapStruct::writeToDisk / readFromDisk,
src/data_struct/map_struct.cu:535-613; DenseMapping::write/readMapFromDisk,
src/voxel_hashing/voxel_hashing.cpp:189-205).

CPU tests run the host-only gbf_dump_write / gbf_dump_read against
tests/golden/ref_dump_small.bin, which the reference's own writer produced
(tests/golden/make_golden.py); the GPU tests dump fused sessions and read them
back into fresh sessions.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import helpers as H
import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
PINS = json.loads((GOLDEN / "reference_pins.json").read_text())["map_dump"]


def pin_blocks():
    """The golden dump's blocks, by the rule pin_main.cu filled them with."""
    pos = np.array(PINS["blocks"], np.int32)
    b = np.arange(len(pos))[:, None]
    i = np.arange(512)[None, :]
    s16 = (((b * 512 + i) * 37) % 65535 - 32767).astype(np.int16)
    sdf = (s16.astype(np.float32) / np.float32(32767)).astype(np.float32)
    w = ((b * 7 + i) % 256).astype(np.float32)
    rgb = np.stack([(b + i) % 256, (b * 3 + i) % 256, (b * 5 + i) % 256], -1).astype(np.uint8)
    return pos, sdf, w, rgb, s16


@pytest.fixture(scope="module")
def L():
    from libfusion_gb300 import build as B
    B.build()
    import libfusion_gb300 as lib
    lib.lib()
    return lib


def test_golden_layout_pins():
    assert PINS["sizeof_voxel"] == O.REF_VOXEL.itemsize == 12
    assert PINS["sizeof_hash_entry"] == O.REF_ENTRY.itemsize == 20
    assert PINS["offsetof_voxel"] == [O.REF_VOXEL.fields[k][1] for k in ("sdf", "weight", "rgb")]
    assert PINS["offsetof_hash_entry"] == [O.REF_ENTRY.fields[k][1] for k in ("ptr", "offset", "pos")]


def test_oracle_reads_golden_through_find_entry():
    d = O.parse_ref_dump(GOLDEN / PINS["file"])
    assert d["size"] == tuple(PINS["size"])
    pos, sdf, w, rgb, s16 = pin_blocks()
    assert int(d["heap_counter"][0]) == PINS["size"][0] - 1 - len(pos)
    for b, p in enumerate(pos):
        i = O.ref_find_entry(d, p)
        assert i >= 0
        ptr = int(d["table"][i]["ptr"])
        vox = d["voxels"][ptr:ptr + 512]
        assert (vox["sdf"] == s16[b]).all() and (vox["weight"] == w[b]).all() and (vox["rgb"] == rgb[b]).all()
    # chains were needed: some blocks live in the excess region
    assert int(d["excess_counter"][0]) > 1


def test_read_golden(L):
    c, s, w, rgb, size = L.read_dump(GOLDEN / PINS["file"])
    assert size == tuple(PINS["size"])
    pos, sdf0, w0, rgb0, _ = pin_blocks()
    c, s, w, rgb = H.sort_blocks(c, s, w, rgb)
    pos, sdf0, w0, rgb0 = H.sort_blocks(pos, sdf0, w0, rgb0)
    np.testing.assert_array_equal(c, pos)
    np.testing.assert_array_equal(s, sdf0)  # int16 / 32767.f, bit for bit
    np.testing.assert_array_equal(w, w0)
    np.testing.assert_array_equal(rgb, rgb0)


def test_write_matches_reference_writer_bytes(L, tmp_path):
    pos, sdf, w, rgb, _ = pin_blocks()
    out = tmp_path / "m.bin"
    L.write_dump(out, pos, sdf, w, rgb, size=tuple(PINS["size"]))
    assert out.read_bytes() == (GOLDEN / PINS["file"]).read_bytes()
    assert Path(str(out) + ".txt").read_bytes() == (GOLDEN / (PINS["file"] + ".txt")).read_bytes()


def test_round_trip_random_blocks(L, tmp_path):
    rng = np.random.default_rng(3)
    pos = np.unique(rng.integers(-3000, 3000, (300, 3)).astype(np.int32), axis=0)
    n = len(pos)
    s16 = rng.integers(-32767, 32768, (n, 512)).astype(np.int16)
    sdf = (s16.astype(np.float32) / np.float32(32767)).astype(np.float32)
    w = rng.integers(0, 256, (n, 512)).astype(np.float32)
    rgb = rng.integers(0, 256, (n, 512, 3)).astype(np.uint8)
    out = tmp_path / "r.bin"
    size = (400, 450, 64)  # 300 blocks in 64 buckets: long excess chains
    L.write_dump(out, pos, sdf, w, rgb, size=size)
    d = O.parse_ref_dump(out)
    assert d["size"] == size
    for b in range(n):  # the reference's own lookup finds every block with its voxels
        i = O.ref_find_entry(d, pos[b])
        assert i >= 0 and int(d["table"][i]["ptr"]) == b * 512
        assert (d["voxels"][b * 512:(b + 1) * 512]["sdf"] == s16[b]).all()
    c2, s2, w2, r2, size2 = L.read_dump(out)
    assert size2 == size
    a = H.sort_blocks(pos, sdf, w, rgb)
    b = H.sort_blocks(c2, s2, w2, r2)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_empty_map_and_default_size(L, tmp_path):
    out = tmp_path / "e.bin"
    z = np.zeros((0, 3), np.int32)
    L.write_dump(out, z, np.zeros((0, 512), np.float32), np.zeros((0, 512), np.float32),
                 np.zeros((0, 512, 3), np.uint8))
    nb, ne, nbk = O.REF_DEFAULT_SIZE
    assert out.stat().st_size == nb * 512 * 12 + ne * 20 + 4 * nb + 4 * nbk + 8
    c, *_, size = L.read_dump(out)
    assert len(c) == 0 and size == O.REF_DEFAULT_SIZE


def test_reader_keeps_first_of_duplicate_entries(L, tmp_path):
    pos, sdf, w, rgb, s16 = pin_blocks()
    raw = bytearray((GOLDEN / PINS["file"]).read_bytes())
    d = O.parse_ref_dump(GOLDEN / PINS["file"])
    nb = PINS["size"][0]
    table = d["table"].copy()
    free = int(np.nonzero(table["ptr"] == -1)[0][-1])
    first = O.ref_find_entry(d, pos[0])
    assert free > first
    table[free] = (11 * 512, 0, tuple(pos[0]))  # a second live entry for block 0's position
    off = nb * 512 * 12
    raw[off:off + table.nbytes] = table.tobytes()
    bad = tmp_path / "dup.bin"
    bad.write_bytes(bytes(raw))
    (tmp_path / "dup.bin.txt").write_bytes((GOLDEN / (PINS["file"] + ".txt")).read_bytes())
    c, s, *_ = L.read_dump(bad)
    assert len(c) == len(pos)
    k = int(np.nonzero((c == pos[0]).all(1))[0][0])
    np.testing.assert_array_equal(s[k], sdf[0])


def test_errors(L, tmp_path):
    pos, sdf, w, rgb, _ = pin_blocks()
    with pytest.raises(L.GbfError, match="CAPACITY"):
        L.write_dump(tmp_path / "a.bin", pos, sdf, w, rgb, size=(8, 24, 8))       # more blocks than the pool
    with pytest.raises(L.GbfError, match="CAPACITY"):
        L.write_dump(tmp_path / "b.bin", pos, sdf, w, rgb, size=(16, 9, 8))       # one excess entry only
    dup = pos.copy()
    dup[3] = dup[1]
    with pytest.raises(L.GbfError, match="INVALID_ARG"):
        L.write_dump(tmp_path / "c.bin", dup, sdf, w, rgb, size=(16, 24, 8))
    with pytest.raises(L.GbfError, match="INVALID_ARG"):
        L.write_dump(tmp_path / "d.bin", pos, sdf, w, rgb, size=(16, 4, 8))      # entries < buckets
    with pytest.raises(L.GbfError, match="IO"):
        L.read_dump(tmp_path / "missing.bin")
    trunc = tmp_path / "t.bin"
    trunc.write_bytes((GOLDEN / PINS["file"]).read_bytes()[:-4])
    (tmp_path / "t.bin.txt").write_bytes((GOLDEN / (PINS["file"] + ".txt")).read_bytes())
    with pytest.raises(L.GbfError, match="IO"):
        L.read_dump(trunc)
    nosize = tmp_path / "n.bin"  # no .txt: the reference's default sizes, which this file does not have
    nosize.write_bytes((GOLDEN / PINS["file"]).read_bytes())
    with pytest.raises(L.GbfError, match="IO"):
        L.read_dump(nosize)
    raw = bytearray((GOLDEN / PINS["file"]).read_bytes())
    off = PINS["size"][0] * 512 * 12
    raw[off:off + 4] = np.int32(17 * 512).tobytes()  # entry 0 points past the 16-block pool
    bad = tmp_path / "p.bin"
    bad.write_bytes(bytes(raw))
    (tmp_path / "p.bin.txt").write_bytes((GOLDEN / (PINS["file"] + ".txt")).read_bytes())
    with pytest.raises(L.GbfError, match="IO"):
        L.read_dump(bad)


# ---- GPU: sessions ---------------------------------------------------------------------------------


def _fused(L, layout, n=4):
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, layout))
    for d, c, T in H.frames(L, K, n, step=3):
        m.update(H.cuda(H.depth_m(d)), H.cuda(c), T)
    return K, m, T


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_session_dump_round_trip(gbf, tmp_path, layout):
    L = gbf
    K, m, T = _fused(L, layout)
    c0, s0, w0, r0 = m.export()
    assert len(c0) > 100
    path = tmp_path / "map.data"
    size = (1 << 15, (1 << 15) + 8192, 1 << 15)
    m.writeMapToDisk(path, size=size)
    d = O.parse_ref_dump(path)
    assert d["size"] == size
    # block i of the export sits at ptr i*512 and the reference's findEntry reaches it
    for b in range(0, len(c0), 7):
        i = O.ref_find_entry(d, c0[b])
        assert i >= 0 and int(d["table"][i]["ptr"]) == b * 512
    vox = d["voxels"][:len(c0) * 512].reshape(len(c0), 512)
    np.testing.assert_array_equal(vox["weight"], w0)
    np.testing.assert_array_equal(vox["rgb"], r0)
    np.testing.assert_array_equal(vox["sdf"], np.trunc(s0 * np.float32(32767)).astype(np.int16))

    m2 = L.DenseMapping(K, H.small_config(L, layout))
    m2.readMapFromDisk(path)
    c1, s1, w1, r1 = m2.export()
    a = H.sort_blocks(c0, s0, w0, r0)
    b = H.sort_blocks(c1, s1, w1, r1)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_array_equal(a[3], b[3])
    if layout != 1:
        np.testing.assert_array_equal(a[1], b[1])  # int16 sdf (REF, SNORM): exact
        # fusing on from the loaded map gives what fusing on from the original gives
        import torch
        d, c, T2 = H.frames(L, K, 1, start=13)[0]
        vm = []
        for mm in (m, m2):
            mm.update(H.cuda(H.depth_m(d)), H.cuda(c), T2)
            v = torch.zeros((K.height, K.width, 4), dtype=torch.float32, device="cuda")
            mm.raycast(v, T2)
            torch.cuda.synchronize()
            vm.append(v.cpu().numpy())
        assert np.isfinite(vm[0]).any()
        np.testing.assert_array_equal(np.nan_to_num(vm[0], nan=7.0), np.nan_to_num(vm[1], nan=7.0))
        a = H.sort_blocks(*m.export())
        b = H.sort_blocks(*m2.export())
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
    else:
        # fp16 sdf -> int16 in the dump -> fp16: one int16 step plus one fp16 rounding
        assert np.abs(a[1] - b[1]).max() <= 1.0 / 32767 + 2.0 ** -11


@pytest.mark.gpu
def test_read_dump_keeps_pose_and_replaces_map(gbf, tmp_path):
    L = gbf
    K, m, T = _fused(L, 0, n=2)
    path = tmp_path / "a.data"
    m.writeMapToDisk(path, size=(1 << 15, (1 << 15) + 4096, 1 << 15))
    s = L.System(K, H.small_config(L, 0))
    d, c, _ = H.frames(L, K, 1, start=40)[0]
    s.process_images(H.cuda(d), H.cuda(c))
    pose = s.get_camera_pose()
    s.readMapFromDisk(path)
    np.testing.assert_array_equal(s.get_camera_pose(), pose)
    a = H.sort_blocks(*m.export())
    b = H.sort_blocks(*s.export())
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.gpu
def test_session_dump_capacity(gbf, tmp_path):
    L = gbf
    K, m, T = _fused(L, 0, n=1)
    n = len(m.export()[0])
    with pytest.raises(L.GbfError, match="CAPACITY"):
        m.writeMapToDisk(tmp_path / "x.data", size=(n - 1, n + 100, 64))
    small = L.DenseMapping(K, H.small_config(L, 0, num_blocks=64))
    m.writeMapToDisk(tmp_path / "y.data", size=(n, n + 4096, 4096))
    with pytest.raises(L.GbfError, match="CAPACITY"):
        small.readMapFromDisk(tmp_path / "y.data")


# ---- GPU: block garbage collection (deleteBlock, map_struct.cu:327-363) -----------------------------


@pytest.mark.gpu
def test_delete_and_prune_blocks(gbf):
    """Deleted blocks leave the map, the others keep their voxels bit for bit, and
    fusing on from the pruned map equals fusing on from a fresh map holding the
    kept blocks (a deleted block that is seen again starts from zero)."""
    import torch
    L = gbf
    K, m, T = _fused(L, 0, n=4)
    c0, s0, w0, r0 = m.export()
    # explicit deletion of every fifth block
    gone = c0[::5]
    assert m.delete_blocks(gone) == len(gone)
    c1, s1, w1, r1 = m.export()
    keep = np.ones(len(c0), bool)
    keep[::5] = False
    a = H.sort_blocks(c0[keep], s0[keep], w0[keep], r0[keep])
    b = H.sort_blocks(c1, s1, w1, r1)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert m.delete_blocks(gone) == 0  # already gone
    # radius prune around the camera centre
    cam = T[:3, 3]
    bm = 8 * m.cfg.voxel_size
    centres = (c1 + 0.5) * bm
    inside = np.linalg.norm(centres - cam, axis=1) <= 1.5
    assert 0 < inside.sum() < len(c1)
    assert m.prune(cam, 1.5) == int((~inside).sum())
    c2, s2, w2, r2 = m.export()
    a = H.sort_blocks(c1[inside], s1[inside], w1[inside], r1[inside])
    b = H.sort_blocks(c2, s2, w2, r2)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    # the same blocks imported into a fresh map fuse on identically
    fresh = L.DenseMapping(K, H.small_config(L, 0))
    fresh.import_blocks(c2, s2, w2, r2)
    d, c, T2 = H.frames(L, K, 1, start=14)[0]
    for mm in (m, fresh):
        mm.update(H.cuda(H.depth_m(d)), H.cuda(c), T2)
    torch.cuda.synchronize()
    a = H.sort_blocks(*m.export())
    b = H.sort_blocks(*fresh.export())
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    # unobserved blocks: a block imported with zero weights is dropped
    z = np.array([[9999, 9999, 9999]], np.int32)
    m.import_blocks(z, np.zeros((1, 512), np.float32), np.zeros((1, 512), np.float32), np.zeros((1, 512, 3), np.uint8))
    n_before = len(m.export()[0])
    assert m.prune(drop_unobserved=True) >= 1
    after = {tuple(x) for x in m.export()[0]}
    assert (9999, 9999, 9999) not in after and len(after) <= n_before - 1


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_collection_of_half_the_blocks_keeps_the_rest_reachable(gbf, layout):
    """A random half of the blocks deleted: many kept blocks sit above the new
    pool end and move into freed positions below it.  The kept blocks keep
    their voxels bit for bit, the pool shrinks to them, the rebuilt table finds
    every kept block (deleting them by list finds them all), and fusing on
    equals fusing on from a fresh map holding the kept blocks."""
    import torch
    L = gbf
    K, m, T = _fused(L, layout, n=4)
    c0, s0, w0, r0 = m.export()
    n0 = len(c0)
    rng = np.random.default_rng(7)
    keep = rng.random(n0) < 0.5
    assert m.delete_blocks(c0[~keep]) == int((~keep).sum())
    assert m.stats().allocated_blocks == int(keep.sum())
    c1, s1, w1, r1 = m.export()
    for x, y in zip(H.sort_blocks(c0[keep], s0[keep], w0[keep], r0[keep]), H.sort_blocks(c1, s1, w1, r1)):
        np.testing.assert_array_equal(x, y)
    fresh = L.DenseMapping(K, H.small_config(L, layout))
    fresh.import_blocks(c1, s1, w1, r1)
    d, c, T2 = H.frames(L, K, 1, start=14)[0]
    for mm in (m, fresh):
        mm.update(H.cuda(H.depth_m(d)), H.cuda(c), T2)
    torch.cuda.synchronize()
    a = H.sort_blocks(*m.export())
    b = H.sort_blocks(*fresh.export())
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    # every block of the map is found in the rebuilt table
    c2 = m.export()[0]
    assert m.delete_blocks(c2) == len(c2) and m.stats().allocated_blocks == 0
