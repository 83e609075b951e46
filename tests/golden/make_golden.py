"""Generate tests/golden/reference_pins.json from the reference's own code.

Builds oracle/ref_pin/build_ref.sh (the reference's map_struct.cu hash and
coordinate converters, voxel.h packing, intrinsic_matrix.h pyramid and
device_tables.h marching-cubes tables, compiled from the reference sources
where they lie) and records its outputs, plus a small map dump written by the
reference's MapStruct::writeToDisk (tests/golden/ref_dump_small.bin + .txt).  The marching-cubes tables are
recorded as SHA-256 digests of their canonical JSON text, so the fixture pins
them without carrying a copy.  Needs the reference tree, so it runs here, not
on the GPU machine; the committed JSON is what the tests read.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]  (default: $LIBFUSION_REFERENCE)
"""
import hashlib
import os
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]


def digest(obj) -> str:
    return hashlib.sha256(json.dumps(obj, separators=(",", ":")).encode()).hexdigest()


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LIBFUSION_REFERENCE", "/root/reference")
    exe = subprocess.run([str(ROOT / "oracle/ref_pin/build_ref.sh"), ref], check=True, capture_output=True,
                         text=True).stdout.strip().splitlines()[-1]
    data = json.loads(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)
    out = {
        "generator": "tests/golden/make_golden.py (oracle/ref_pin/pin_main.cu + reference map_struct.cu)",
        "hash": data["hash"],
        "voxel_block_local": data["voxel_block_local"],
        "world_to_voxel": data["world_to_voxel"],
        "pack_sdf": data["pack_sdf"],
        "intrinsics_pyr": data["intrinsics_pyr"],
        "edge_table_sha256": digest(data["edge_table"]),
        "triangle_table_sha256": digest(data["triangle_table"]),
        "triangle_counts": [sum(1 for v in row if v != -1) // 3 for row in data["triangle_table"]],
    }
    # the reference's own MapStruct::writeToDisk on a small chained map (pin_main.cu dump_pin)
    dump = ROOT / "tests/golden/ref_dump_small.bin"
    lines = subprocess.run([exe, "dump", str(dump)], check=True, capture_output=True, text=True).stdout.splitlines()
    out["map_dump"] = json.loads(next(l for l in lines if l.startswith("{")))
    out["map_dump"]["file"] = dump.name
    dst = ROOT / "tests/golden/reference_pins.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {dst}")


if __name__ == "__main__":
    main()
