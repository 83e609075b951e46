"""TUM RGB-D frame source (TUMLoader, src/input/tum_loader.cpp:7-64): the
association-file parsing, the PNG codec (every row filter of the PNG
specification, 8 and 16 bits) and the TUM -> millimetre depth conversion; on
the GPU, a sequence written in TUM form fuses exactly like the frames it holds."""
import zlib
import struct

import numpy as np
import pytest

import helpers as H
from libfusion_gb300 import tum


def _filtered_png(path, img):
    """Encode with row filter y % 5 (None, Sub, Up, Average, Paeth), computed
    straight from the PNG specification's definitions."""
    h, w = img.shape[:2]
    ch = 1 if img.ndim == 2 else img.shape[2]
    depth = 16 if img.dtype == np.uint16 else 8
    raw = (img.astype(">u2") if depth == 16 else img).tobytes()
    bpp = ch * depth // 8
    stride = w * bpp
    rows = [raw[y * stride:(y + 1) * stride] for y in range(h)]
    out = bytearray()
    prev = bytes(stride)
    for y, row in enumerate(rows):
        f = y % 5
        enc = bytearray(stride)
        for x in range(stride):
            a = row[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            enc[x] = (row[x] - pred) & 0xFF
        out += bytes([f]) + enc
        prev = row
    ctype = {1: 0, 3: 2, 4: 6}[ch]

    def chunk(k, p):
        return struct.pack(">I", len(p)) + k + p + struct.pack(">I", zlib.crc32(k + p))

    path.write_bytes(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)) +
                     chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b""))


@pytest.mark.parametrize("shape,dtype", [((13, 17), np.uint16), ((13, 17, 3), np.uint8), ((9, 11, 4), np.uint8),
                                         ((10, 7), np.uint8)])
def test_png_round_trip_all_filters(tmp_path, shape, dtype):
    rng = np.random.default_rng(1)
    img = rng.integers(0, np.iinfo(dtype).max, shape, endpoint=True).astype(dtype)
    _filtered_png(tmp_path / "f.png", img)
    np.testing.assert_array_equal(tum.read_png(tmp_path / "f.png"), img)
    tum.write_png(tmp_path / "w.png", img)
    np.testing.assert_array_equal(tum.read_png(tmp_path / "w.png"), img)


def test_png_rejects_bad_files(tmp_path):
    (tmp_path / "x.png").write_bytes(b"not a png")
    with pytest.raises(ValueError):
        tum.read_png(tmp_path / "x.png")


def test_association_and_depth_units(tmp_path):
    rng = np.random.default_rng(2)
    d_mm = rng.integers(0, 6000, (4, 6), endpoint=True).astype(np.uint16)
    c = rng.integers(0, 256, (4, 6, 3)).astype(np.uint8)
    (tmp_path / "depth").mkdir()
    (tmp_path / "rgb").mkdir()
    lines = []
    for k in range(3):
        tum.write_png(tmp_path / f"depth/{k}.png", (d_mm.astype(np.uint32) * 5 + k).astype(np.uint16))
        tum.write_png(tmp_path / f"rgb/{k}.png", c)
        lines.append(f"{100 + k}.5 depth/{k}.png {100 + k}.25 rgb/{k}.png")
    (tmp_path / "association.txt").write_text("\n".join(lines) + "\n")
    ld = tum.TUMLoader(tmp_path)
    assert ld.images_loaded == 3 and ld.time_stamps == [100.25, 101.25, 102.25]  # the colour timestamps
    for k in range(3):
        assert ld.has_images()
        d, img = ld.get_next_images()
        np.testing.assert_array_equal(img, c)
        # TUM units (5000 per metre) -> millimetres, rounded
        np.testing.assert_array_equal(tum.depth_mm(d), np.rint((d_mm * 5.0 + k) / 5.0).astype(np.uint16))
    assert not ld.has_images() and ld.get_next_images() is None
    with pytest.raises(FileNotFoundError):
        tum.TUMLoader(tmp_path / "missing")


@pytest.mark.gpu
def test_tum_sequence_fuses_like_its_frames(gbf, tmp_path):
    """Frames written as a TUM sequence (depth x5 in TUM units) and read back
    give bit-identical poses and maps to processing the frames directly."""
    import torch
    L = gbf
    K = H.intrinsics(L)
    fr = H.frames(L, K, 4, step=2)
    (tmp_path / "d").mkdir()
    (tmp_path / "c").mkdir()
    lines = []
    for k, (d, c, _) in enumerate(fr):
        tum.write_png(tmp_path / f"d/{k}.png", (d.astype(np.uint32) * 5).astype(np.uint16))
        tum.write_png(tmp_path / f"c/{k}.png", c)
        lines.append(f"{k}.0 d/{k}.png {k}.0 c/{k}.png")
    (tmp_path / "association.txt").write_text("\n".join(lines))
    a, b = L.System(K, H.small_config(L, 1)), L.System(K, H.small_config(L, 1))
    a.set_pose(fr[0][2])
    b.set_pose(fr[0][2])
    ld = tum.TUMLoader(tmp_path)
    for d, c, _ in fr:
        a.process_images(H.cuda(d), H.cuda(c))
        dt, ct = ld.get_next_images()
        b.process_images(H.cuda(tum.depth_mm(dt)), H.cuda(ct))
    torch.cuda.synchronize()
    assert np.array_equal(a.get_camera_pose(), b.get_camera_pose())
    for x, y in zip(H.sort_blocks(*a.export()), H.sort_blocks(*b.export())):
        assert np.array_equal(x, y)
