#!/bin/sh
# Compile the reference's integration, z-range / raycast, ICP-row,
# photometric-row, image (derivative, back-projection, normals, shading) and
# marching-cubes kernels (src/voxel_hashing/depth_fusion.cu, ray_tracing.cu,
# scene_mesh.cu, src/tracking/cuda_imgproc.cu,
# src/tracking/pose_estimator.cu, m_estimator.cu, with src/data_struct/
# map_struct.cu for the map state, read where they lie under the reference
# tree) into device modules for sm_103a, with the pin entry points of
# oracle/ref_pin/pin_*.cu and the OpenCV / Sophus stand-ins of
# oracle/ref_pin/stub_cv.  Output only into oracle/_ref/.
#   pin_<name>.cubin       -fmad=false: every float operation rounded as
#                          written, the arithmetic the oracle restates
#   pin_<name>_fmad.cubin  nvcc's default contraction, as the reference's own
#                          CMake build would compile it (for the record)
# Usage: oracle/ref_pin/build_kernels.sh [REFERENCE_ROOT]  (default: $LIBFUSION_REFERENCE, else /root/reference)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${LIBFUSION_REFERENCE:-/root/reference}}
OUT="$HERE/../_ref"
mkdir -p "$OUT"
FLAGS="-cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -w --expt-relaxed-constexpr -I $REF/include -I $REF -I $HERE/stub_cv -I $HERE"
pids=""
for m in fusion raycast icp rgb imgproc mesh; do
    nvcc $FLAGS -fmad=false "$HERE/pin_$m.cu" -o "$OUT/pin_$m.cubin" & pids="$pids $!"
    nvcc $FLAGS "$HERE/pin_$m.cu" -o "$OUT/pin_${m}_fmad.cubin" & pids="$pids $!"
done
rc=0
for p in $pids; do wait $p || rc=1; done
exit $rc
