"""The oracle pinned against outputs of the reference's own code
(tests/golden/reference_pins.json, generated by tests/golden/make_golden.py
from src/data_struct/map_struct.cu, include/data_struct/voxel.h,
include/data_struct/intrinsic_matrix.h and include/voxel_hashing/device_tables.h)."""
import ctypes as C
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_pins.json").read_text())


def digest(obj) -> str:
    return hashlib.sha256(json.dumps(obj, separators=(",", ":")).encode()).hexdigest()


def test_compute_hash_matches_reference(oracle_lib):
    # computeHash (map_struct.cu:143-148), int32 wraparound included
    bad = [(x, y, z, n, h) for x, y, z, n, h in GOLD["hash"] if oracle_lib.or_compute_hash(x, y, z, n) != h]
    assert not bad, bad[:5]
    assert len(GOLD["hash"]) > 4000


def test_voxel_block_local_match_reference(oracle_lib):
    for row in GOLD["voxel_block_local"]:
        v = (C.c_int * 3)(*row[:3])
        b, l = (C.c_int * 3)(), (C.c_int * 3)()
        oracle_lib.or_voxel_to_block(v, b)
        oracle_lib.or_voxel_to_local(v, l)
        assert list(b) == row[3:6], row
        assert list(l) == row[6:9], row
        assert oracle_lib.or_local_idx(l) == row[9]


def test_world_to_voxel_matches_reference(oracle_lib):
    # worldPtToVoxelPos: pt / voxel (true float division), then ToVector3i
    for x, v, rx, ry, rz in GOLD["world_to_voxel"]:
        x32, v32 = np.float32(x), np.float32(v)
        p = (x32, -x32, np.float32(x32 * np.float32(0.5)))
        got = [oracle_lib.or_floor_ref(float(np.float32(c / v32))) for c in p]
        assert got == [rx, ry, rz], (x, v, got)


def test_sdf_packing_matches_reference(oracle_lib):
    for s, packed, unpacked, weight in GOLD["pack_sdf"]:
        assert oracle_lib.or_pack_sdf(s) == packed
        assert np.float32(oracle_lib.or_unpack_sdf(packed)) == np.float32(unpacked)
        assert weight == 255.0  # setWeight clamps at 255


def test_marching_cubes_tables_match_reference(oracle_lib):
    edge = [oracle_lib.or_edge_table(i) for i in range(256)]
    assert digest(edge) == GOLD["edge_table_sha256"]
    tri = []
    for i in range(256):
        out = (C.c_int * 16)()
        n = oracle_lib.or_tri_table(i, out)
        assert n // 3 == GOLD["triangle_counts"][i]
        tri.append(list(out))
    assert digest(tri) == GOLD["triangle_table_sha256"]


def test_product_table_is_the_oracle_table():
    """The CUDA source carries the same packed table as the oracle."""
    root = Path(__file__).resolve().parents[1]
    inc = (root / "oracle" / "mc_table.inc").read_text().split()
    src = (root / "libfusion_gb300" / "csrc" / "mesh.cu").read_text()
    body = src[src.index("kTriPacked[256] = {") + len("kTriPacked[256] = {"):]
    body = body[:body.index("};")].split()
    assert body == inc


def test_intrinsics_pyramid_matches_reference():
    # IntrinsicMatrix::pyr_down halves every field in float (intrinsic_matrix.h:33-37)
    w, h, fx, fy, cx, cy = 640, 480, np.float32(525), np.float32(525), np.float32(319.5), np.float32(239.5)
    for row in GOLD["intrinsics_pyr"]:
        assert [w, h] == row[:2]
        assert [fx, fy, cx, cy] == [np.float32(v) for v in row[2:6]]
        assert np.float32(1) / fx == np.float32(row[6])
        s = np.float32(0.5)
        w, h = int(s * np.float32(w)), int(s * np.float32(h))
        fx, fy, cx, cy = s * fx, s * fy, s * cx, s * cy


def test_jtjjtr_packing_order():
    # create_jtjjtr (reduce_sum.h:48-61): i <= j < 7 row-major upper triangle,
    # j == 6 goes to Jtr, [27] = sum r^2, [28] = count
    idx = {}
    k = 0
    for i in range(7):
        for j in range(i, 7):
            idx[(i, j)] = k
            k += 1
    assert k == 28 and idx[(6, 6)] == 27 and idx[(0, 6)] == 6 and idx[(5, 6)] == 26
