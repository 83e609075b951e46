// Reference-kernel pin module: z-range tiles and the raycast march
// (src/voxel_hashing/ray_tracing.cu).  The functors are called the way the
// reference's call_device_functor kernels call them (include/utils/
// safe_call.h:31-35), with create_rendering_blocks' and raycast's launch
// shapes chosen by the caller (1024-thread CTAs over the visible blocks, then
// 16x16 CTAs 4 per row of rendering blocks; 4x8 CTAs over the pixels).
#include "src/data_struct/map_struct.cu"
#include "src/voxel_hashing/ray_tracing.cu"
#include "pin_common.cuh"

namespace pin {
__device__ inline fusion::cuda::RenderingBlockDelegate rendering_delegate(
    int width, int height, const float *inv_pose, float fx, float fy, float cx, float cy, unsigned *count,
    unsigned n_visible, fusion::HashEntry *visible, float *zx, float *zy, int zcols, int zrows,
    fusion::RenderingBlock *blocks) {
    fusion::cuda::RenderingBlockDelegate d;
    d.width = width;
    d.height = height;
    d.inv_pose = m34(inv_pose);
    d.fx = fx;
    d.fy = fy;
    d.cx = cx;
    d.cy = cy;
    d.rendering_block_count = count;
    d.visible_block_count = n_visible;
    d.visible_block_pos = visible;
    d.zrange_x = cv::cuda::PtrStepSz<float>(zrows, zcols, zx, (size_t)zcols * sizeof(float));
    d.zrange_y = cv::cuda::PtrStep<float>(zy, (size_t)zcols * sizeof(float));
    d.rendering_blocks = blocks;
    return d;
}
}  // namespace pin

// create_rendering_blocks (ray_tracing.cu:223-277): the list pass ...
extern "C" __global__ void pin_rendering_blocks(int width, int height, const float *inv_pose, float fx, float fy,
                                                float cx, float cy, unsigned *count, unsigned n_visible,
                                                fusion::HashEntry *visible, float *zx, float *zy, int zcols,
                                                int zrows, fusion::RenderingBlock *blocks) {
    const auto d = pin::rendering_delegate(width, height, inv_pose, fx, fy, cx, cy, count, n_visible, visible, zx, zy,
                                           zcols, zrows, blocks);
    d();
}

// ... and the fill pass
extern "C" __global__ void pin_fill_rendering_blocks(int width, int height, const float *inv_pose, float fx, float fy,
                                                     float cx, float cy, unsigned *count, unsigned n_visible,
                                                     fusion::HashEntry *visible, float *zx, float *zy, int zcols,
                                                     int zrows, fusion::RenderingBlock *blocks) {
    const auto d = pin::rendering_delegate(width, height, inv_pose, fx, fy, cx, cy, count, n_visible, visible, zx, zy,
                                           zcols, zrows, blocks);
    d.fill_rendering_blocks();
}

// raycast (ray_tracing.cu:577-609): MapRenderingDelegate::operator()
extern "C" __global__ void pin_raycast(fusion::Voxel *voxels, fusion::HashEntry *table, float *vmap, int width,
                                       int height, const float *zx, const float *zy, int zcols, int zrows,
                                       float invfx, float invfy, float cx, float cy, const float *pose,
                                       const float *inv_pose) {
    fusion::cuda::MapRenderingDelegate d;
    d.width = width;
    d.height = height;
    d.map_struct.heap_mem_ = nullptr;
    d.map_struct.excess_counter_ = nullptr;
    d.map_struct.heap_mem_counter_ = nullptr;
    d.map_struct.bucket_mutex_ = nullptr;
    d.map_struct.voxels_ = voxels;
    d.map_struct.hash_table_ = table;
    d.vmap = cv::cuda::PtrStep<fusion::Vector4f>((fusion::Vector4f *)vmap, (size_t)width * 16);
    d.zrange_x = cv::cuda::PtrStepSz<float>(zrows, zcols, (float *)zx, (size_t)zcols * sizeof(float));
    d.zrange_y = cv::cuda::PtrStepSz<float>(zrows, zcols, (float *)zy, (size_t)zcols * sizeof(float));
    d.invfx = invfx;
    d.invfy = invfy;
    d.cx = cx;
    d.cy = cy;
    d.pose = pin::m34(pose);
    d.inv_pose = pin::m34(inv_pose);
    d();
}
