#!/bin/sh
# Compile the reference's own hash / coordinate / voxel-packing / table code
# (src/data_struct/map_struct.cu and headers, read where they lie under the
# reference tree) with the pin program.  Output only into oracle/_ref/.
# Usage: oracle/ref_pin/build_ref.sh [REFERENCE_ROOT]  (default: $LIBFUSION_REFERENCE, else /root/reference)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${LIBFUSION_REFERENCE:-/root/reference}}
OUT="$HERE/../_ref"
mkdir -p "$OUT"
nvcc -std=c++14 -O0 -rdc=true -I "$REF/include" -I "$HERE/stub" \
    "$HERE/pin_main.cu" "$REF/src/data_struct/map_struct.cu" -o "$OUT/ref_pin"
echo "$OUT/ref_pin"
