// gbf_kernels.h -- host-side launchers of the sm_103a kernels.
//
// Every launcher takes the device array of SessionView for `nslots` slots and
// the largest image extent among them; slots whose `active` is 0 return at once.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbfusion.h"
#include "gbf_types.h"

namespace gbf {

struct Extent {
    int w, h;        // largest level-0 size among the slots
    int max_pool;    // largest block pool among the slots
    int max_red[kMaxLevels]; // largest reduction CTA count per level
    int levels;      // largest level count
    int max_iter[kMaxLevels];
    int ray_tw;      // raycast tile width (4, 8, 16 or 32 of a 64-pixel tile); 0 = 8
};

inline int ray_tile_width(const Extent &ex) {
    return (ex.ray_tw == 4 || ex.ray_tw == 16 || ex.ray_tw == 32) ? ex.ray_tw : 8;
}

// ---- ingest (ingest.cu) ------------------------------------------------------
struct IngestArgs {
    int set_sel;                 // 0: current set (1-idx), 1: reference set (idx)
    int src;                     // 0: staging u16+rgb8, 1: external u16, 2: external float
    const void *depth; long long depth_pitch;
    const uint8_t *rgb; long long rgb_pitch;
};
void launch_ingest(const SessionView *d_sv, int nslots, const Extent &ex, const IngestArgs &a, cudaStream_t st);

// ---- mapping (mapping.cu) ------------------------------------------------------
struct FuseImport {
    const float *depth; long long depth_pitch;
    const uint8_t *rgb; long long rgb_pitch;
    const float *nmap; long long nmap_pitch;
};
// mode: 0 colour update (1/d^2), 1 weighted update with the reference set's
// level-0 normals, 2 weighted update with the imported normals.
void launch_fuse_import(const SessionView *d_sv, const Extent &ex, const FuseImport &in, cudaStream_t st);
void launch_fuse(const SessionView *d_sv, int nslots, const Extent &ex, int mode, const int *layouts,
                 cudaStream_t st);
void launch_alloc_visible(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st);
// visible list = allocated blocks in the frustum of the map pose (no fuse)
void launch_visible_frustum(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st);
// Phong shading of camera-frame vertex / normal maps into RGBA8 (rgb NULL = untextured)
void launch_render(const float4 *vmap, long long vmap_pitch, const float4 *nmap, long long nmap_pitch,
                   const uint8_t *rgb, long long rgb_pitch, int rgb_stride, int w, int h, uchar4 *out,
                   long long out_pitch, cudaStream_t st);
void launch_integrate(const SessionView *d_sv, int nslots, const Extent &ex, int mode, const int *layouts,
                      cudaStream_t st);

// ---- raycast (raycast.cu) -------------------------------------------------------
// rgb_ext (optional): the hits' nearest voxel colours, 3 bytes per pixel, white elsewhere
void launch_raycast(const SessionView *d_sv, int nslots, const Extent &ex, float4 *vmap_ext, long long vmap_pitch,
                    int post_pyramid, const int *layouts, cudaStream_t st, uint8_t *rgb_ext = nullptr,
                    long long rgb_pitch = 0);
void launch_zrange(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st);
void launch_march(const SessionView *d_sv, int nslots, const Extent &ex, float4 *vmap_ext, long long vmap_pitch,
                  const int *layouts, cudaStream_t st, uint8_t *rgb_ext = nullptr, long long rgb_pitch = 0);
// computeNMapK (cuda_imgproc.cu:276-305) of a pitched vertex map into a pitched normal map
void launch_nmap_of(const float4 *vmap, long long vmap_pitch, float4 *nmap, long long nmap_pitch, int w, int h,
                    cudaStream_t st);
// kernel launches of one launch_post
int post_launches(const Extent &ex);
void launch_post(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st);

// ---- tracking (tracking.cu) -----------------------------------------------------
// mode 0: full Gauss-Newton (gbf_track / process frame), stops at the schedule end
// kernel launches of one launch_track over nslots sessions
int track_launches(int nslots, const Extent &ex);
void launch_track(const SessionView *d_sv, int nslots, const Extent &ex, int frame_mode, cudaStream_t st);
// single reduction for gbf_reduce: pose given as float 3x4 in the kernel args
void launch_reduce_once(const SessionView *d_sv, const Extent &ex, int level, const float *pose12, float stddev,
                        cudaStream_t st);
// frame bookkeeping after tracking: pose update, reference swap
void launch_frame_finish(const SessionView *d_sv, int nslots, cudaStream_t st);
// per-slot pose / tracking / status record of a batch tick (empty slots zero)
void launch_slot_results(const SessionView *d_sv, int nslots, gbf_slot_result *out, cudaStream_t st);

// ---- meshing (mesh.cu) ------------------------------------------------------------
// returns via device counters; the host reads C_MESH_TRIS
void launch_mesh(const SessionView *d_sv, const Extent &ex, int layout, int mode, float *vtx, void *attr,
                 long long max_tris, int *counts, cudaStream_t st);

}  // namespace gbf
