// Shared helpers of the reference-kernel pin modules (oracle/ref_pin/pin_*.cu).
// Test infrastructure: each module is the reference's own translation unit,
// included where it lies, plus extern "C" entry points that set the
// reference's __device__ MapState and call its device functors the way its
// host functions do.  Built by oracle/ref_pin/build_kernels.sh into
// oracle/_ref/*.cubin; never part of the product.
#pragma once

namespace pin {

// fusion::Matrix3x4f from 12 row-major floats (the float cast of a pose, as
// Sophus::SE3d::cast<float>().matrix3x4() gives it)
__device__ inline fusion::Matrix3x4f m34(const float *p) {
    fusion::Matrix3x4f m;
    m.R0 = fusion::Vector4f(p[0], p[1], p[2], p[3]);
    m.R1 = fusion::Vector4f(p[4], p[5], p[6], p[7]);
    m.R2 = fusion::Vector4f(p[8], p[9], p[10], p[11]);
    return m;
}

}  // namespace pin

// The reference keeps its map parameters in one __device__ MapState
// (src/data_struct/map_struct.cu:10), uploaded by MapStruct's constructor.
extern "C" __global__ void pin_set_state(int num_buckets, int num_entries, int num_blocks, float voxel_size,
                                         float zmin_raycast, float zmax_raycast, float zmin_update,
                                         float zmax_update, int max_rendering_blocks, int max_mesh_triangles) {
    fusion::MapState s;
    s.num_total_buckets_ = num_buckets;
    s.num_total_hash_entries_ = num_entries;
    s.num_total_voxel_blocks_ = num_blocks;
    s.num_max_mesh_triangles_ = max_mesh_triangles;
    s.num_max_rendering_blocks_ = max_rendering_blocks;
    s.zmin_raycast = zmin_raycast;
    s.zmax_raycast = zmax_raycast;
    s.zmin_update = zmin_update;
    s.zmax_update = zmax_update;
    s.voxel_size = voxel_size;
    fusion::param = s;
}

// The values the reference derives from the state (map_struct.cu:100-128):
// out = {truncation_dist, inverse_voxel_size, raycast_step_scale, block_size_metric}
extern "C" __global__ void pin_state_values(float *out) {
    out[0] = fusion::param.truncation_dist();
    out[1] = fusion::param.inverse_voxel_size();
    out[2] = fusion::param.raycast_step_scale();
    out[3] = fusion::param.block_size_metric();
}

// sizeof of the reference's device records as this module compiles them:
// out = {Voxel, HashEntry, RenderingBlock, MapState}
extern "C" __global__ void pin_sizes(int *out) {
    out[0] = (int)sizeof(fusion::Voxel);
    out[1] = (int)sizeof(fusion::HashEntry);
    out[2] = (int)sizeof(fusion::RenderingBlock);
    out[3] = (int)sizeof(fusion::MapState);
}
