// gbf_types.h -- data layout shared by the host runtime and the sm_103a kernels.
//
// One session = one reconstruction (the reference's DenseMapping + DenseOdometry
// pair).  All of its state lives in one device arena; the kernels see it through
// a SessionView (plain pointers and parameters).  Every kernel is written over a
// *batch* of sessions: blockIdx.y selects the slot, so the single-session
// ("plain") path is a batch of one and the served path runs many sessions per
// launch.  Replaces the reference's single process-global `__device__ MapState
// param` (src/data_struct/map_struct.cu:10), which allowed one map per process.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbf {

constexpr int kMaxLevels = 5;
constexpr int kNumLayouts = 3;         // gbf_voxel_layout values
constexpr int kBlockSide = 8;
constexpr int kBlockVoxels = 512;
constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kCoordBits = 21;          // per block coordinate in the packed key
constexpr int kCoordLimit = 1 << 20;    // |block coordinate| must stay below this
constexpr int kReduceThreads = 256;     // CTA size of the ICP/RGB reduction
constexpr int kReducePixelsPerThread = 4;
// pixels per reduction CTA on the pyramid levels above the finest (level 0
// takes kReduceThreads * kReducePixelsPerThread)
constexpr int kCoarseReduceTile = 1024;
constexpr int kReduceWidth = 58;        // 29 ICP + 29 RGB sums
constexpr int kPartialStride = 64;      // floats per CTA partial record

// Open-addressing hash slot.  key packs the block position (21 bits per axis,
// two's complement), ptr is the pool block id (-1 while unassigned).  The home
// slot is the reference's computeHash (map_struct.cu:143-148) modulo the slot
// count, probed linearly.
struct __align__(16) HashSlot {
    unsigned long long key;
    int ptr;
    int pad;
};

struct LevelK {
    int w, h;
    float fx, fy, cx, cy, invfx, invfy;
};

// Per-session device counters.
enum Counter {
    C_NUSED = 0,      // blocks taken from the pool (may exceed pool on exhaustion)
    C_NVIS = 1,       // visible blocks of the last fuse
    C_STATUS = 2,     // GBF_FLAG_* bits
    C_FRAME = 3,      // fuse counter (allocation stamp)
    C_RENDER = 4,     // renderable blocks of the last z-range pass
    C_TICKET = 5,     // last-CTA-done ticket of the reduction
    C_MESH_BLOCKS = 6,
    C_MESH_TRIS = 7,
    C_GC_DELETED = 8, // blocks deleted by the last garbage collection
    C_COUNT = 16
};

// Tracking and pose state of a session, resident on the device.
struct TrackState {
    double pose[12];       // T_wc of the newest frame (3x4 row-major)
    double map_pose[12];   // pose used by fuse / raycast
    float map_twc[12];     // map_pose and its inverse rounded to float (the reference's
    float map_tcw[12];     // pose.cast<float>() / pose.inverse().cast<float>())
    double est[12];        // Revertable<SE3d> current (icp_tracker.cpp:25)
    double est_prev[12];   // Revertable<SE3d> previous
    double init[12];       // initial estimate of the current tracking run
    double update[12];     // TrackingResult::update
    float icp_error, rgb_error, stddev;
    int icp_count, rgb_count;
    int level_done;        // the `break` of the current level
    int invalid;           // invalid_error
    int iterations;
    int has_ref;           // a reference image set exists
    int idx;               // which image set (0/1) is the reference
    int success;
    int tracking;          // this frame runs Gauss-Newton
    float icp_inliers, rgb_inliers;
    long long frame_index;
    long long pixel_iterations;   // cumulative pixels reduced by Gauss-Newton iterations
    long long integrated_blocks;  // cumulative visible blocks integrated
    int level_iters[kMaxLevels];  // iterations run per level in the last tracking
    double last_sums[kReduceWidth];
};

struct SessionView {
    int active;
    int layout;            // gbf_voxel_layout
    int cap, pool, max_probe;
    int motion_prior;      // gbf_config::motion_prior
    int cap_mask;          // cap - 1 when cap is a power of two, else -1
    float voxel, inv_voxel, tau, inv_tau, step_scale;
    float zmin_u, zmax_u, zmin_r, zmax_r, block_metric;
    float w_icp, w_rgb, icp_dist, icp_angle;
    int bilateral;
    int levels;
    int max_iter[kMaxLevels];
    LevelK lv[kMaxLevels];
    int red_ctas[kMaxLevels];   // reduction CTAs per level
    int red_tile[kMaxLevels];   // reference pixels per reduction CTA per level

    // map
    HashSlot *table;
    int4 *bcoord;          // per pool block: x, y, z, slot
    int *bstamp;           // fuse counter of the last touch
    unsigned char *bfresh; // 1 = voxels not yet initialised
    void *vox_sw;          // sdf + weight word per voxel, 512 per block: HALF uint32
                           // (fp16 sdf | fp16 weight << 16), REF uint2 (int16 sdf, f32 weight)
    uchar4 *vox_rgb;
    int *vis;              // visible block ids
    int *ctr;              // Counter array

    // images (dense, pitch = width)
    uint16_t *in_depth;    // staging u16 mm
    uint8_t *in_rgb;       // staging rgb8
    float *depth_raw;      // level-0 metres, unfiltered (fused)
    uchar4 *rgb4;          // level-0 colour (fused)
    float4 *nmap_ext;      // imported normal map (gbf_fuse)
    float2 *fuse_px;       // per pixel of the fused frame: (depth or NaN if rejected, weight)
    float *depth[kMaxLevels];
    float *inten[2][kMaxLevels];
    float *gx[kMaxLevels];
    float *gy[kMaxLevels];
    // per set and level, (I, dI/dx, dI/dy, 0) of each pixel: one 16-byte gather per
    // bilinear tap of the photometric row instead of three 4-byte ones (null: not kept)
    float4 *igd[2][kMaxLevels];
    float4 *vmap[2][kMaxLevels];
    float4 *nmap[2][kMaxLevels];
    float *zr_min, *zr_max;
    int zr_w, zr_h;

    TrackState *ts;
    float *partials;       // [red_ctas][kPartialStride]
    int *mesh_off;         // per-block triangle counts / offsets (pool + 1)
};

}  // namespace gbf
