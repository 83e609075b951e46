"""TUM RGB-D sequences (TUMLoader, src/input/tum_loader.cpp:7-64 of the reference).

Host-side frame source for the fusion path: ``association.txt`` in the sequence
root lists ``<depth timestamp> <depth file> <colour timestamp> <colour file>`` per
line (the reference reads the two file names in that order and keeps the
second timestamp); the images are 16-bit depth PNGs in TUM units (5000 per
metre) and 8-bit colour PNGs.  With no image library in this environment the
PNGs are decoded here (zlib inflate + the five PNG row filters; non-interlaced
grey / RGB / RGBA, 8 or 16 bits).

Two reference behaviours are not copied: ``cv::imread`` returns the colour in
BGR order, which the reference then converts to grey as if it were RGB; and
``System::process_images`` scales every depth image by 1/1000
(src/system.cpp:43), so TUM depth would reach it five times too far.  Here the
colour stays RGB and ``depth_mm`` converts TUM units to millimetres, the unit of
``System.process_images``.
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

TUM_DEPTH_FACTOR = 5000.0  # TUM depth PNG units per metre

_PNG_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 6: 4}  # colour type -> samples per pixel


def _paeth(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    p = a.astype(np.int32) + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c)).astype(np.uint8)


def read_png(path) -> np.ndarray:
    """Decode a non-interlaced 8/16-bit grey, RGB or RGBA PNG into (H, W[, C])."""
    data = Path(path).read_bytes()
    if data[:8] != _PNG_SIG:
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if hdr is None:
        raise ValueError(f"{path}: no IHDR chunk")
    w, h, depth, ctype, _, _, interlace = hdr
    if depth not in (8, 16) or ctype not in _CHANNELS or interlace != 0:
        raise ValueError(f"{path}: unsupported PNG (bit depth {depth}, colour type {ctype}, interlace {interlace})")
    ch = _CHANNELS[ctype]
    bpp = ch * depth // 8  # bytes per pixel: the filters' left neighbour distance
    stride = w * bpp
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    if raw.size != h * (stride + 1):
        raise ValueError(f"{path}: image data has {raw.size} bytes, expected {h * (stride + 1)}")
    rows = raw.reshape(h, stride + 1)
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.uint8)
    for y in range(h):
        f, line = rows[y, 0], rows[y, 1:]
        if f == 0:
            cur = line.copy()
        elif f == 2:
            cur = line + prev
        else:
            cur = np.zeros(stride, np.uint8)
            if f == 1:  # Sub: a running sum per byte lane, modulo 256
                cur = (np.cumsum(line.reshape(-1, bpp).astype(np.uint32), axis=0) & 0xFF).astype(np.uint8).ravel()
            elif f == 3:
                for x0 in range(0, stride, bpp):
                    left = cur[x0 - bpp:x0].astype(np.uint16) if x0 else np.zeros(bpp, np.uint16)
                    cur[x0:x0 + bpp] = line[x0:x0 + bpp] + ((left + prev[x0:x0 + bpp]) // 2).astype(np.uint8)
            elif f == 4:
                for x0 in range(0, stride, bpp):
                    left = cur[x0 - bpp:x0] if x0 else np.zeros(bpp, np.uint8)
                    ul = prev[x0 - bpp:x0] if x0 else np.zeros(bpp, np.uint8)
                    cur[x0:x0 + bpp] = line[x0:x0 + bpp] + _paeth(left, prev[x0:x0 + bpp], ul)
            else:
                raise ValueError(f"{path}: bad filter type {f} in row {y}")
        out[y] = cur
        prev = cur
    if depth == 16:
        img = out.view(">u2").astype(np.uint16).reshape(h, w, ch)
    else:
        img = out.reshape(h, w, ch)
    return img[..., 0] if ch == 1 else img


def write_png(path, img: np.ndarray) -> None:
    """Encode (H, W) uint8/uint16 grey or (H, W, 3|4) uint8 as a PNG (filter 0)."""
    img = np.ascontiguousarray(img)
    if img.ndim == 2:
        ctype, ch = 0, 1
    elif img.ndim == 3 and img.shape[2] in (3, 4):
        ctype, ch = (2, 3) if img.shape[2] == 3 else (6, 4)
    else:
        raise ValueError("expected (H, W), (H, W, 3) or (H, W, 4)")
    if img.dtype == np.uint16:
        depth, body = 16, img.astype(">u2").tobytes()
    elif img.dtype == np.uint8:
        depth, body = 8, img.tobytes()
    else:
        raise ValueError("expected uint8 or uint16 samples")
    h, w = img.shape[:2]
    stride = w * ch * depth // 8
    rows = np.frombuffer(body, np.uint8).reshape(h, stride)
    raw = np.concatenate([np.zeros((h, 1), np.uint8), rows], axis=1).tobytes()

    def chunk(kind: bytes, payload: bytes) -> bytes:
        return struct.pack(">I", len(payload)) + kind + payload + struct.pack(">I", zlib.crc32(kind + payload))

    Path(path).write_bytes(_PNG_SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)) +
                           chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def depth_mm(depth_tum: np.ndarray, factor: float = TUM_DEPTH_FACTOR) -> np.ndarray:
    """TUM depth units -> uint16 millimetres (rounded; 0 stays 0 = no measurement)."""
    mm = np.rint(depth_tum.astype(np.float64) * (1000.0 / factor))
    return np.clip(mm, 0, 65535).astype(np.uint16)


class TUMLoader:
    """TUMLoader (tum_loader.h:10-28): frames of a TUM sequence in association order."""

    def __init__(self, root_path):
        self.root_path = Path(root_path)
        self.image_id = 0
        self.time_stamps: list[float] = []
        self.depth_filenames: list[str] = []
        self.image_filenames: list[str] = []
        self.load_association()

    @property
    def images_loaded(self) -> int:
        return len(self.depth_filenames)

    def load_association(self) -> bool:
        """association.txt: `ts depth_file ts image_file` per line (tum_loader.cpp:34-64)."""
        f = self.root_path / "association.txt"
        if not f.exists():
            raise FileNotFoundError(f"cannot locate the association file {f}")
        tokens = f.read_text().split()
        for i in range(0, len(tokens) - 3, 4):
            _, fd, ts, fi = tokens[i:i + 4]
            self.depth_filenames.append(fd)
            self.image_filenames.append(fi)
            self.time_stamps.append(float(ts))
        if not self.depth_filenames:
            raise ValueError(f"TUM loading failed: no frames in {f}")
        return True

    def has_images(self) -> bool:
        return self.image_id < self.images_loaded

    def get_next_images(self):
        """(depth in TUM units (H, W) uint16, colour (H, W, 3) uint8 RGB), or None at the end."""
        if not self.has_images():
            return None
        depth = read_png(self.root_path / self.depth_filenames[self.image_id])
        image = read_png(self.root_path / self.image_filenames[self.image_id])
        if image.ndim == 3 and image.shape[2] == 4:
            image = image[..., :3]
        self.image_id += 1
        return depth, np.ascontiguousarray(image)
