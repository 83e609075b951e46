/*
 * gbfusion.h -- C ABI of libgbfusion, the GB300 (sm_103a) dense RGB-D fusion
 * hot path: voxel-hashed TSDF mapping (allocation, visible-block enumeration,
 * integration, raycast, marching cubes) and point-to-plane ICP + photometric
 * tracking over image pyramids.
 *
 * Every entry point returns a gbf_status; on failure gbf_last_error() gives a
 * message (thread-local).  No entry point exits the process (the reference's
 * safe_call does exit(0), include/utils/safe_call.h:13-23).
 *
 * Images are device pointers with a row pitch in BYTES.  Poses are 4x4
 * row-major double matrices T_wc (camera -> world), the matrix form of the
 * reference's Sophus::SE3d frame poses.  `stream` is a cudaStream_t passed as
 * void* (NULL = legacy default stream).
 *
 * Threading: a session is driven from one host thread at a time (calls on the
 * same session are not synchronised); different sessions may be used from
 * different threads concurrently.  A batch is internally synchronised: its
 * calls may come from several threads -- camera threads staging frames while
 * one thread runs the ticks and reads the results -- and each holds the batch's
 * lock for its duration (gbf_batch_process and gbf_batch_results may wait
 * there for an earlier tick).  A session in a batch is driven through the batch
 * while it sits there; it must outlive its slot (gbf_batch_set(b, slot, NULL)
 * or gbf_batch_destroy before gbf_session_destroy).
 *
 * Mapping of reference interfaces (paths relative to the reference project):
 *   DenseMapping::DenseMapping(K)          include/voxel_hashing/voxel_hashing.h:15   -> gbf_session_create
 *   DenseMapping::update(frame)            src/voxel_hashing/voxel_hashing.cpp:44-65  -> gbf_fuse (nmap given)
 *   DenseMapping::update(depth,image,pose) src/voxel_hashing/voxel_hashing.cpp:67-85  -> gbf_fuse (nmap NULL)
 *   DenseMapping::raycast                  src/voxel_hashing/voxel_hashing.cpp:87-119 -> gbf_raycast
 *   DenseMapping::raycast_check_visibility src/voxel_hashing/voxel_hashing.cpp:121-135 -> gbf_raycast_check_visibility
 *   renderScene / renderSceneTextured      src/tracking/cuda_imgproc.cu:50-108        -> gbf_render_scene, gbf_session_render
 *   DenseMapping::reset_mapping            src/voxel_hashing/voxel_hashing.cpp:137-140 -> gbf_session_reset
 *   DenseMapping::fetch_mesh_*             src/voxel_hashing/voxel_hashing.cpp:142-187 -> gbf_extract_mesh
 *   DenseMapping::write/readMapFromDisk    src/voxel_hashing/voxel_hashing.cpp:189-205 -> gbf_map_write_dump / gbf_map_read_dump
 *   MapStruct::writeToDisk/readFromDisk    src/data_struct/map_struct.cu:535-613      -> gbf_dump_write / gbf_dump_read
 *   DeviceImage::upload                    src/tracking/device_image.cpp:146-181      -> gbf_build_pyramid
 *   DenseTracking::compute_transform       src/tracking/icp_tracker.cpp:23-156        -> gbf_track
 *   icp_reduce / rgb_step                  src/tracking/pose_estimator.cu:267-307,
 *                                          src/tracking/m_estimator.cu:437-482        -> gbf_reduce
 *   System::process_images                 src/system.cpp:40-114                      -> gbf_process_frame
 */
#ifndef GBFUSION_H
#define GBFUSION_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GBF_API __attribute__((visibility("default")))
#else
#define GBF_API
#endif

#define GBF_MAX_LEVELS 5
#define GBF_BLOCK_SIDE 8
#define GBF_BLOCK_VOXELS 512

typedef enum gbf_status {
    GBF_OK = 0,
    GBF_ERR_INVALID_ARG = 1,  /* bad pointer, size or configuration          */
    GBF_ERR_CUDA = 2,         /* a CUDA runtime call failed                   */
    GBF_ERR_OUT_OF_MEMORY = 3,/* device allocation failed                     */
    GBF_ERR_CAPACITY = 4,     /* batch slot / output buffer too small         */
    GBF_ERR_NO_DEVICE = 5,    /* no CUDA device visible                       */
    GBF_ERR_IO = 6            /* a file could not be opened, read or written, or
                                 its contents are not a valid map dump          */
} gbf_status;

/* Per-session device status bits (sticky until gbf_session_reset). */
enum {
    GBF_FLAG_POOL_EXHAUSTED = 1u << 0, /* block pool full: blocks were not allocated */
    GBF_FLAG_HASH_FULL      = 1u << 1, /* probe limit hit: blocks were not allocated */
    GBF_FLAG_COORD_RANGE    = 1u << 2, /* block coordinate outside +-2^20            */
    GBF_FLAG_TRACK_FAILED   = 1u << 3, /* a frame's tracking failed since the reset
                                          (pose kept for it); the last frame's result
                                          is gbf_frame_stats.track.success          */
    GBF_FLAG_NAN_POSE       = 1u << 4  /* solver produced a non-finite pose          */
};

typedef enum gbf_voxel_layout {
    GBF_VOXEL_REF = 0,  /* int16 sdf (x32767, truncating) + f32 weight (<=255) + rgb8:
                           the reference Voxel semantics, include/data_struct/voxel.h:11-66 */
    GBF_VOXEL_HALF = 1, /* fp16 sdf + 16-bit weight (binary16, <=255) + rgb8: 8 B per voxel */
    GBF_VOXEL_SNORM = 2 /* int16 sdf (packed as sdf x 32767 rounded to nearest, unpacked as
                           code x 0x1.000202p-15f, 1/32767 rounded up) + 16-bit weight (binary16,
                           <=255) + rgb8: 8 B per voxel, a uniform 3.1e-5 sdf step where fp16's
                           step grows to 4.9e-4 near +-1 */
} gbf_voxel_layout;

typedef enum gbf_mesh_mode {
    GBF_MESH_VERTEX = 0, /* fetch_mesh_vertex_only  */
    GBF_MESH_NORMAL = 1, /* fetch_mesh_with_normal  */
    GBF_MESH_COLOUR = 2  /* fetch_mesh_with_colour  */
} gbf_mesh_mode;

/* IntrinsicMatrix, include/data_struct/intrinsic_matrix.h:12-20 (invfx/invfy derived). */
typedef struct gbf_intrinsics {
    int32_t width, height;
    float fx, fy, cx, cy;
} gbf_intrinsics;

/* MapState (include/data_struct/map_struct.h:17-51) + TrackingContext
 * (include/tracking/icp_tracker.h:20-26) + the thresholds the reference
 * hard-codes (pose_estimator.cu:292-293, icp_tracker.cpp:89-90). */
typedef struct gbf_config {
    float voxel_size;     /* metres                                               */
    float truncation;     /* metres (reference hard-codes 5*voxel_size)           */
    float zmin_update, zmax_update, zmin_raycast, zmax_raycast;
    int32_t num_buckets;  /* hash slots (power of two not required)               */
    int32_t num_blocks;   /* block pool size                                      */
    int32_t voxel_layout; /* gbf_voxel_layout                                     */
    int32_t num_levels;   /* pyramid levels, 1..GBF_MAX_LEVELS                    */
    int32_t max_iterations[GBF_MAX_LEVELS]; /* per level, level 0 = finest         */
    float w_icp, w_rgb;   /* A = w_icp*H_icp + w_rgb*H_rgb (reference: 1e6, 1)    */
    float icp_dist_thresh;  /* metres (reference 0.01)                            */
    float icp_angle_thresh; /* compared with |n_c x n_l| (reference cos(30*3.14/180)) */
    int32_t bilateral;    /* 1: bilateral-filter the tracking depth (reference)   */
    int32_t max_probe;    /* hash probe limit (bounded insert/lookup)             */
    int32_t motion_prior; /* 0: a frame's tracking starts from no motion (the reference,
                             rgbd_odometry.cpp:33-37); 1: from the last frame's motion
                             when that frame tracked (constant velocity), else none  */
} gbf_config;

typedef struct gbf_track_result {
    int32_t success;      /* TrackingResult::sucess                               */
    int32_t iterations;   /* Gauss-Newton iterations actually run                 */
    float icp_error, rgb_error;
    float icp_inliers, rgb_inliers; /* correspondences of the last iteration       */
    double update[16];    /* TrackingResult::update (T_ref<-cur), row-major 4x4   */
} gbf_track_result;

typedef struct gbf_frame_stats {
    int64_t frame_index;
    int32_t allocated_blocks;
    int32_t visible_blocks;
    int32_t render_blocks_valid;
    uint32_t status;      /* GBF_FLAG_* bits                                      */
    gbf_track_result track;
    int32_t level_iterations[GBF_MAX_LEVELS]; /* last tracking, per level          */
    int64_t pixel_iterations;  /* cumulative pixels x Gauss-Newton iterations     */
    int64_t integrated_blocks; /* cumulative visible blocks integrated            */
} gbf_frame_stats;

typedef struct gbf_session gbf_session;
typedef struct gbf_batch gbf_batch;
typedef struct gbf_synth_scene gbf_synth_scene;

/* ---- library ---------------------------------------------------------------- */
GBF_API const char *gbf_version(void);
GBF_API const char *gbf_last_error(void);
/* Fills the reference's MapStruct defaults (src/data_struct/map_struct.cu:17-35),
 * with truncation = 5*voxel as MapState::truncation_dist (map_struct.cu:120-123),
 * a 3-level 10/5/3 pyramid and the reference tracking thresholds. */
GBF_API gbf_status gbf_config_default(gbf_config *cfg);
/* Device bytes one session needs (admission control); host-only, no GPU. */
GBF_API gbf_status gbf_session_bytes(const gbf_config *cfg, const gbf_intrinsics *K, uint64_t *bytes);

/* ---- session: DenseMapping + DenseOdometry state on one GPU ---------------- */
GBF_API gbf_status gbf_session_create(const gbf_config *cfg, const gbf_intrinsics *K, gbf_session **out);
GBF_API gbf_status gbf_session_destroy(gbf_session *s);
GBF_API gbf_status gbf_session_reset(gbf_session *s, void *stream);
/* Device input staging buffers owned by the session (u16 depth in mm, pitch
 * width*2; rgb8 packed, pitch width*3), filled by the caller before
 * gbf_process_frame_staged / gbf_batch_process. */
GBF_API gbf_status gbf_session_inputs(gbf_session *s, uint16_t **depth_mm_dev, uint8_t **rgb_dev);
/* Copy one frame (host -- pinned for an asynchronous copy -- or device memory)
 * into the session's staging buffers on `stream`. */
GBF_API gbf_status gbf_session_stage(gbf_session *s, const uint16_t *depth_mm, int64_t depth_pitch,
                                     const uint8_t *rgb, int64_t rgb_pitch, void *stream);
GBF_API gbf_status gbf_set_pose(gbf_session *s, const double T_wc[16], void *stream);
GBF_API gbf_status gbf_get_pose(gbf_session *s, double T_wc[16], void *stream);
GBF_API gbf_status gbf_get_stats(gbf_session *s, gbf_frame_stats *out, void *stream);

/* ---- mapping ------------------------------------------------------------------ */
/* Allocate blocks along every valid pixel's truncation band, enumerate visible
 * blocks and integrate TSDF + colour.  depth: float metres (rows 4-byte aligned).
 * rgb: 3 bytes/px.  nmap (float4, rows 16-byte aligned) != NULL selects the
 * normal-weighted update (update_map_weighted_kernel,
 * depth_fusion.cu:356-428), NULL the 1/d^2 update (update_map_with_colour_kernel,
 * depth_fusion.cu:288-354). */
GBF_API gbf_status gbf_fuse(gbf_session *s, const float *depth_dev, int64_t depth_pitch,
                            const uint8_t *rgb_dev, int64_t rgb_pitch,
                            const float *nmap_dev, int64_t nmap_pitch,
                            const double T_wc[16], void *stream);
/* z-range tiles from the last fuse's visible blocks, then a per-pixel raycast
 * into vmap (float4 per pixel, NaN = no hit; rows 16-byte aligned).  As in the
 * reference, vmap is left untouched when the last fuse saw no visible /
 * renderable block. */
GBF_API gbf_status gbf_raycast(gbf_session *s, const double T_wc[16],
                               float *vmap_dev, int64_t vmap_pitch, void *stream);
/* gbf_raycast plus, when given, the model normals and colours:
 *   nmap (float4 per pixel, rows 16-byte aligned): computeNMapK
 *     (src/tracking/cuda_imgproc.cu:276-305) of the vertex map, the normals the
 *     reference's next frame tracks against;
 *   rgb (3 bytes per pixel): the colour raycast_with_colour
 *     (src/voxel_hashing/ray_tracing.cu:478-564) means to write -- a hit's nearest
 *     voxel colour (read_colour, :427-441), white where there is no hit or that
 *     voxel is unobserved.  (The reference's host call runs the plain raycast
 *     instead and writes no colour; the vertex map here keeps the plain raycast's
 *     hits.) */
GBF_API gbf_status gbf_raycast_maps(gbf_session *s, const double T_wc[16], float *vmap_dev, int64_t vmap_pitch,
                                    float *nmap_dev, int64_t nmap_pitch, uint8_t *rgb_dev, int64_t rgb_pitch,
                                    void *stream);
/* DenseMapping::raycast_check_visibility (src/voxel_hashing/voxel_hashing.cpp:121-135):
 * the visible-block list recomputed for pose T by the frustum test alone
 * (count_visible_entry, src/voxel_hashing/ray_tracing.cu:778-807) over every
 * allocated block, then gbf_raycast at T -- a raycast from any pose, e.g. for
 * relocalisation.  The list replaces the last fuse's, as in the reference. */
GBF_API gbf_status gbf_raycast_check_visibility(gbf_session *s, const double T[16], float *vmap, int64_t vmap_pitch,
                                                void *stream);
/* renderScene / renderSceneTextured (src/tracking/cuda_imgproc.cu:50-108): Phong
 * shading of a camera-frame vertex and normal map (float4, pitched) into RGBA8,
 * light at (5, 5, 5) in the camera frame; rgb8 (pitched) textures it, NULL =
 * white.  Device pointers. */
GBF_API gbf_status gbf_render_scene(const float *vmap, int64_t vmap_pitch, const float *nmap, int64_t nmap_pitch,
                                    const uint8_t *rgb, int64_t rgb_pitch, int32_t width, int32_t height,
                                    uint8_t *out, int64_t out_pitch, void *stream);
/* DeviceImage::get_rendered_image / get_rendered_scene_textured
 * (src/tracking/device_image.cpp:119-129): the session's model prediction (the
 * level-0 vertex and normal maps of its last raycast) shaded; textured with the
 * last fused frame's colour. */
GBF_API gbf_status gbf_session_render(gbf_session *s, int32_t textured, uint8_t *out, int64_t out_pitch,
                                      void *stream);
/* Marching cubes over all allocated blocks into caller-allocated device
 * buffers (3 float3 per triangle; attr: 3 float3 normals or 3 uchar3 colours).
 * *n_tris receives the triangle count clamped to max_tris (synchronises). */
GBF_API gbf_status gbf_extract_mesh(gbf_session *s, int32_t mode, float *vertex_dev, void *attr_dev,
                                    uint64_t max_tris, uint64_t *n_tris, void *stream);

/* ---- tracking ----------------------------------------------------------------- */
/* Build the intensity / vertex / normal pyramids of a frame into the session's
 * `current` image set (which=0) or `reference` set (which=1). */
GBF_API gbf_status gbf_build_pyramid(gbf_session *s, int32_t which, const float *depth_dev, int64_t depth_pitch,
                                     const uint8_t *rgb_dev, int64_t rgb_pitch, void *stream);
/* One ICP + photometric reduction at `level` for pose T (T_cur<-ref, float
 * cast as the reference) and photometric stddev: out[0..28] ICP sums, out[29..57]
 * RGB sums in the create_jtjjtr packing (reduce_sum.h:48-61). Synchronises. */
GBF_API gbf_status gbf_reduce(gbf_session *s, int32_t level, const double T[16], float stddev,
                              double out[58], void *stream);
/* Level-0 images of a reference and a current frame, owned by the caller (dense
 * rows; vertex / normal maps float4 per pixel, intensities and gradients float).
 * The vertex and normal maps and the reference intensity start on 16-byte
 * boundaries, the other images on 4-byte boundaries (GBF_ERR_INVALID_ARG
 * otherwise); nothing past an image's last pixel is read, so the images may sit
 * back to back in one buffer. */
typedef struct gbf_reduce_inputs {
    int32_t width, height;
    float fx, fy, cx, cy;
    const float *ref_vmap, *ref_nmap, *ref_intensity;
    const float *cur_vmap, *cur_nmap, *cur_intensity, *cur_didx, *cur_didy;
    float dist_thresh, angle_thresh;
} gbf_reduce_inputs;
/* No counterpart in the reference: the same 58 sums as gbf_reduce, for callers
 * that cannot allocate device memory -- real-time loops that forbid allocation
 * once they run, and frameworks that hand out all device memory through their
 * own allocator.  Needs no session and calls no cudaMalloc / cudaFree: its
 * scratch (per-CTA partials + a ticket) is a fixed 512 KB array in the library
 * that every GPU loading the library keeps until exit.  Images up to 2,097,152
 * pixels (larger ones return GBF_ERR_CAPACITY).  out_dev: 58 doubles of device
 * memory, 8-byte aligned, written on `stream`.  The first call on a device
 * looks the array's address up (make it before any stream capture); calls that
 * overlap on the GPU share the array and race. */
GBF_API gbf_status gbf_reduce_noalloc(const gbf_reduce_inputs *in, const double T[16], float stddev,
                                      double *out_dev, void *stream);
/* Coarse-to-fine Gauss-Newton between the reference and current sets. Synchronises. */
GBF_API gbf_status gbf_track(gbf_session *s, const double init[16], gbf_track_result *out, void *stream);
/* Copy one pyramid image: kind 0 vmap, 1 nmap (float4), 2 intensity, 3 dI/dx,
 * 4 dI/dy, 5 filtered depth (float). which: 0 current, 1 reference. */
GBF_API gbf_status gbf_get_image(gbf_session *s, int32_t which, int32_t kind, int32_t level,
                                 void *out_dev, int64_t pitch, void *stream);

/* ---- full frame: System::process_images -------------------------------------- */
/* ingest (u16 mm -> m, rgb -> gray, pyramids) -> track against the model
 * prediction -> fuse raw depth at the new pose -> raycast the new reference
 * vertex map -> rebuild its pyramid.  No host synchronisation. */
GBF_API gbf_status gbf_process_frame(gbf_session *s, const uint16_t *depth_mm_dev, int64_t depth_pitch,
                                     const uint8_t *rgb_dev, int64_t rgb_pitch, void *stream);
/* Same, from the session's own staging buffers (gbf_session_inputs). */
GBF_API gbf_status gbf_process_frame_staged(gbf_session *s, void *stream);

/* ---- map export / import (canonical per-block form) ---------------------------- */
/* Allocated blocks: coords[3*i] block position, sdf/weight float per voxel
 * (512 per block, index z*64+y*8+x), rgb 3 bytes per voxel.  Synchronises. */
GBF_API gbf_status gbf_map_export(gbf_session *s, int32_t *coords, float *sdf, float *weight, uint8_t *rgb,
                                  int64_t max_blocks, int64_t *n_blocks);
GBF_API gbf_status gbf_map_import(gbf_session *s, const int32_t *coords, const float *sdf, const float *weight,
                                  const uint8_t *rgb, int64_t n_blocks);
/* ---- map dump in the reference's raw layout ------------------------------------ */
/* MapSize (include/data_struct/map_struct.h:53-58): the three sizes a dump is
 * laid out with.  The reference's own writer always uses its MapState
 * defaults (src/data_struct/map_struct.cu:19-21): 200000 blocks, 250000 hash
 * entries (200000 buckets + 50000 excess). */
typedef struct gbf_map_size {
    int32_t num_blocks;
    int32_t num_hash_entries;
    int32_t num_buckets;
} gbf_map_size;

/* File layout, as MapStruct::writeToDisk writes it (src/data_struct/map_struct.cu:535-573):
 *   Voxel[num_blocks*512]      12 B: int16 sdf (x32767, truncated), 2 pad, float weight,
 *                              uint8 rgb[3], 1 pad           (include/data_struct/voxel.h:20-22)
 *   HashEntry[num_hash_entries] 20 B: int32 ptr (block id * 512, -1 empty), int32 offset
 *                              (1-based excess link), int32 pos[3] (include/data_struct/hash_entry.h:20-22)
 *   int32 heap[num_blocks], int32 bucket_mutex[num_buckets], int32 heap_counter, int32 excess_counter
 * and "<path>.txt" holds the MapSize as three raw int32.
 *
 * gbf_dump_write / gbf_dump_read are host-only (no device, no session): they
 * convert between that layout and the canonical per-block arrays of
 * gbf_map_export / gbf_map_import.  The writer lays blocks out as the
 * reference's single-threaded createBlock (map_struct.cu:280-323) would after
 * inserting them in the given order: block i at ptr i*512, home bucket
 * computeHash(pos, num_buckets) when free, else appended to that bucket's
 * excess chain with offsets 1, 2, ... in insertion order; the heap and its
 * counter as after i pops; excess_counter = the next free offset.  (The
 * reference's first excess insert takes offset 0, which links nothing and
 * lands on bucket num_buckets-1; the writer does not reproduce that.)
 * The reader takes every entry with ptr != -1, in table order, as the
 * reference's visibility pass does (src/voxel_hashing/depth_fusion.cu:49-93);
 * a position seen twice keeps its first entry.  sdf = int16 / 32767.f. */
GBF_API gbf_status gbf_dump_write(const char *path, const gbf_map_size *size, const int32_t *coords,
                                  const float *sdf, const float *weight, const uint8_t *rgb, int64_t n_blocks);
/* With coords == NULL only *size and *n_blocks are filled. */
GBF_API gbf_status gbf_dump_read(const char *path, gbf_map_size *size, int32_t *coords, float *sdf, float *weight,
                                 uint8_t *rgb, int64_t max_blocks, int64_t *n_blocks);
/* DenseMapping::writeMapToDisk (src/voxel_hashing/voxel_hashing.cpp:189-196): the
 * session's allocated blocks, in block-id order, through gbf_dump_write.
 * size NULL = the reference's default sizes.  Synchronises. */
GBF_API gbf_status gbf_map_write_dump(gbf_session *s, const char *path, const gbf_map_size *size);
/* DenseMapping::readMapFromDisk (src/voxel_hashing/voxel_hashing.cpp:198-205): replaces
 * the session's map with the dump's blocks; the camera pose and tracking state
 * are kept, as in the reference, which uploads only the map storage.
 * Synchronises. */
GBF_API gbf_status gbf_map_read_dump(gbf_session *s, const char *path);

/* ---- session snapshot: evict to host memory, resume --------------------------- */
/* No counterpart in the reference, which keeps one map per process and dumps only
 * its map storage (MapStruct::writeToDisk, src/data_struct/map_struct.cu:534-613).
 * A snapshot holds what a session's next frame reads: its allocated blocks in the
 * session's own voxel layout (block ids kept), its pose and tracking state (the
 * motion prior included), its counters and status bits, and the reference frame's
 * pyramid (the raycast prediction's vertex and normal maps, the intensities).
 * Restored into a session created with the same configuration and intrinsics (and
 * the same library version), the session continues exactly as the original would
 * have: the same poses and the same map, bit for bit.  Take a snapshot between
 * frames (for a staggered batch, after gbf_batch_flush); dst / src may be host or
 * device memory.  All three synchronise: snapshot_bytes with the whole device,
 * snapshot and restore with `stream`, which must be ordered after the session's
 * last frame. */
GBF_API gbf_status gbf_session_snapshot_bytes(gbf_session *s, int64_t *bytes);
/* *written (may be NULL) = the snapshot's size; GBF_ERR_CAPACITY when capacity is smaller. */
GBF_API gbf_status gbf_session_snapshot(gbf_session *s, void *dst, int64_t capacity, int64_t *written,
                                        void *stream);
/* GBF_ERR_INVALID_ARG when src is not a snapshot of this library version, or was
 * taken from a session of another configuration or intrinsics. */
GBF_API gbf_status gbf_session_restore(gbf_session *s, const void *src, int64_t bytes, void *stream);

/* ---- block garbage collection ------------------------------------------------- */
/* deleteBlock (src/data_struct/map_struct.cu:327-363) for a list of blocks: their
 * voxels and table entries go, the pool is compacted (the kept blocks above the
 * new pool end move into the freed positions below it) and the table is
 * rebuilt from the kept blocks, all on the device.  The reference defines
 * deleteBlock but never calls it (its one caller is commented out,
 * depth_fusion.cu:70), so its pool only grows; a long-running session prunes
 * here.  A deleted block that is observed again starts from zero, as a block
 * the reference re-creates would.  Pose and tracking state are kept; the last
 * fuse's visible list is emptied (its block ids no longer hold).  Blocks not
 * in the map are ignored.  Synchronises; *n_deleted (may be NULL) = blocks
 * removed. */
GBF_API gbf_status gbf_map_delete_blocks(gbf_session *s, const int32_t *coords, int64_t n, int64_t *n_deleted);
/* Delete the blocks whose centre lies farther than `radius` metres from
 * `center` (world frame; center NULL or radius < 0: no distance test) and, with
 * drop_unobserved, the blocks without any observed voxel (all weights 0).
 * Synchronises; *n_deleted (may be NULL) = blocks removed. */
GBF_API gbf_status gbf_map_prune(gbf_session *s, const double center[3], double radius, int32_t drop_unobserved,
                                 int64_t *n_deleted);
/* gbf_map_prune enqueued on `stream` with no host synchronisation and no
 * allocation, for a serving loop that collects between frames: a handful of
 * launches in the session's stream order (after its last frame's fusion, before
 * its next).  The count is not returned; gbf_get_stats gives the blocks left. */
GBF_API gbf_status gbf_map_prune_async(gbf_session *s, const double center[3], double radius,
                                       int32_t drop_unobserved, void *stream);

/* Visible-block list of the last fuse (block coordinates), synchronises. */
GBF_API gbf_status gbf_visible_blocks(gbf_session *s, int32_t *coords, int64_t max_blocks, int64_t *n_blocks);
/* z-range grid of the last raycast: 2 floats per cell (min, max), (H/8)x(W/8). */
GBF_API gbf_status gbf_zrange(gbf_session *s, float *out_host, int64_t max_cells);

/* ---- batch: many sessions per launch ----------------------------------------- */
GBF_API gbf_status gbf_batch_create(int32_t max_sessions, gbf_batch **out);
/* Destroying a batch frees it: no other gbf_batch_* call on it may be pending
 * on another thread, or start, once gbf_batch_destroy begins (the batch's lock
 * cannot outlive the batch). */
GBF_API gbf_status gbf_batch_destroy(gbf_batch *b);
GBF_API gbf_status gbf_batch_set(gbf_batch *b, int32_t slot, gbf_session *s);
/* No counterpart in the reference (one map per process there).  Reserve the
 * tick's shape for up to `slots` slots of sessions no larger than (cfg, K):
 * frame size, pyramid, iteration counts, block pool and voxel layout.  The
 * captured tick depends only on that shape, so with a reservation, sessions
 * of up to that size put into and taken out of slots below `slots` (serving
 * admission and eviction) keep the captured graphs and the tuner's choice;
 * launches are sized for the reservation, and smaller sessions' surplus
 * CTAs return at once.  slots = 0 drops the reservation. */
GBF_API gbf_status gbf_batch_reserve(gbf_batch *b, const gbf_config *cfg, const gbf_intrinsics *K, int32_t slots);
/* One frame for every slot with active[slot] != 0, from each session's staging
 * buffers, all sessions in the same launches; replayed from a CUDA graph when
 * use_graph != 0 (captured on first use for the current slot assignment). */
GBF_API gbf_status gbf_batch_process(gbf_batch *b, const uint8_t *active, int32_t use_graph, void *stream);
/* Read slot `slot`'s next frames straight from device buffers (dense u16 depth
 * and rgb8 of the session's size) instead of its staging buffers; the pointers
 * are taken at each gbf_batch_process call (NULL, NULL restores staging). */
GBF_API gbf_status gbf_batch_set_inputs(gbf_batch *b, int32_t slot, const uint16_t *depth_dev, const uint8_t *rgb_dev);
/* Copy slot `slot`'s frame for the NEXT gbf_batch_process from host (or
 * device) memory into the batch's own input buffers, on `stream`.  The buffers
 * are double-buffered by tick parity: the copy waits on the device for the
 * tick two submissions back (the last reader of that parity), and the next
 * gbf_batch_process waits on the device for the copy, so frames for tick k+1
 * can be staged on a copy stream while tick k runs.  A staged frame is used by
 * one tick (then the slot falls back to set_inputs / the session's staging). */
GBF_API gbf_status gbf_batch_stage(gbf_batch *b, int32_t slot, const uint16_t *depth, int64_t depth_pitch,
                                   const uint8_t *rgb, int64_t rgb_pitch, void *stream);
/* Per-slot outcome of a tick, copied to pinned host memory at the end of every tick. */
typedef struct gbf_slot_result {
    double pose[16];      /* camera -> world after the tick, row-major 4x4          */
    int32_t tracked;      /* the tick's tracking succeeded (TrackingResult::sucess) */
    uint32_t status;      /* GBF_FLAG_* bits                                         */
    int64_t frame_index;  /* frames the session has processed                       */
} gbf_slot_result;
/* Results of the last submitted tick (back = 0) or the one before (back = 1):
 * waits for that tick, then copies min(n, slots) records.  Reading tick k-1
 * after submitting tick k keeps the device busy while the host reads. */
GBF_API gbf_status gbf_batch_results(gbf_batch *b, int32_t back, gbf_slot_result *out, int32_t n);
/* Concurrent session groups per tick (1..4, default 2): the slots are split
 * into contiguous groups whose frames run as parallel branches of the tick
 * (graph branches / forked streams).  Results do not depend on it. */
GBF_API gbf_status gbf_batch_set_groups(gbf_batch *b, int32_t groups);
/* Staggered groups (default off; with 2+ groups): the odd groups run half a
 * frame out of phase -- each tick they fuse and raycast their previous frame,
 * then ingest and track the new one -- so one group's tracking shares the GPU
 * with the other's fusion and raycast.  Each session still runs every step in
 * order and every result is the same; the poses in gbf_batch_results are those
 * of the tick's frames, while an odd group's map holds the previous frame until
 * the next tick or gbf_batch_flush. */
GBF_API gbf_status gbf_batch_set_stagger(gbf_batch *b, int32_t enable);
/* Raycast tile of the batch's ticks: 64 pixels, tile_w (4, 8, 16 or 32) wide;
 * default 8 (8x8).  Results do not depend on it. */
GBF_API gbf_status gbf_batch_set_ray_tile(gbf_batch *b, int32_t tile_w);

/* Online autotuner of the tick's launch shape: session groups (1..4), stagger
 * (with 2+ groups) and the raycast tile.  These knobs change how a tick is
 * launched, never what it computes, so the batch tunes while it serves: each
 * candidate gets ticks_per_candidate ticks, timed with CUDA events on the
 * submitting stream (the first tick after a switch, which captures a new graph,
 * is not timed).  The search tries groups x stagger at the 8-wide tile, then the
 * tile widths at the best of those, and keeps the fastest median.  The choice is
 * recorded in a process-wide table under the batch's shape (device, slot count,
 * largest frame size, pool, pyramid and iteration counts, voxel layouts); a batch
 * of a recorded shape settles from it at its next tick, without exploring, and a
 * change of shape (gbf_batch_set with another size) looks up or explores again.
 * Setting groups, stagger or the tile by hand turns the tuner off. */
#define GBF_TUNE_MAX_REPORT 16
typedef struct gbf_launch_shape {
    int32_t groups, stagger, ray_tile_w;
    float median_ms; /* median timed tick (0: not timed) */
} gbf_launch_shape;
typedef struct gbf_tuning {
    int32_t state;                /* 0 off, 1 exploring, 2 settled                  */
    int32_t from_table;           /* settled from the process-wide table            */
    int32_t ticks_per_candidate;
    gbf_launch_shape chosen;      /* the shape in use                               */
    int32_t n_tried;              /* candidates timed so far (this batch)          */
    gbf_launch_shape tried[GBF_TUNE_MAX_REPORT];
} gbf_tuning;
GBF_API gbf_status gbf_batch_set_autotune(gbf_batch *b, int32_t enable, int32_t ticks_per_candidate);
GBF_API gbf_status gbf_batch_tuning(gbf_batch *b, gbf_tuning *out);
/* Clear the process-wide table of tuned shapes. */
GBF_API gbf_status gbf_autotune_forget(void);
/* Fuse and raycast what the staggered groups owe, and wait: call before reading
 * a batched session's map (export, mesh, raycast) or driving it alone.  Changing
 * the slots, groups, stagger or timing, and destroying the batch, flush too. */
GBF_API gbf_status gbf_batch_flush(gbf_batch *b, void *stream);
/* Record CUDA events at the phase boundaries of every tick (captured into the
 * graph): ingest, track, alloc+visible, integrate, z-range, march, post. */
GBF_API gbf_status gbf_batch_set_timing(gbf_batch *b, int32_t enable);
/* Mean durations (ms) of the 7 phases over the ticks since timing was enabled
 * (waits for the outstanding ticks); ms[7], when n > 7, receives the tick count. */
GBF_API gbf_status gbf_batch_phase_ms(gbf_batch *b, float *ms, int32_t n);
/* Number of kernel launches one tick makes. */
GBF_API gbf_status gbf_batch_kernels(gbf_batch *b, int32_t *n);
/* Tick graphs the batch has captured so far (one per tick parity for each tick
 * shape; a change of shape, groups, stagger, tile or timing drops them).  A
 * server watches it to see that admissions and evictions do not re-capture. */
GBF_API gbf_status gbf_batch_captures(gbf_batch *b, int64_t *n);

/* ---- synthetic RGB-D scenes (test and benchmark input) ------------------------ */
typedef struct gbf_synth_params {
    float room[3];       /* box room extent x, y, z (metres); z up            */
    int32_t n_spheres, n_boxes;
    float sphere_rmin, sphere_rmax;
    uint64_t seed;
    int32_t trajectory;  /* 0 circle (r, height, yaw jitter), 1 figure-eight   */
    float radius, height, yaw_jitter_deg, speed; /* speed in m/s for figure-eight */
    float fps;
    int32_t frames_per_loop;
    float noise;         /* 1 = depth noise sigma 0.0012+0.0019(z-0.4)^2, 0 = none */
    float zclip_min, zclip_max;
} gbf_synth_params;

GBF_API gbf_status gbf_synth_default(gbf_synth_params *p);
GBF_API gbf_status gbf_synth_create(const gbf_synth_params *p, gbf_synth_scene **out);
GBF_API gbf_status gbf_synth_destroy(gbf_synth_scene *sc);
GBF_API gbf_status gbf_synth_pose(const gbf_synth_scene *sc, int32_t frame, double T_wc[16]);
GBF_API gbf_status gbf_synth_render(const gbf_synth_scene *sc, const gbf_intrinsics *K, const double T_wc[16],
                                    int32_t frame, uint16_t *depth_mm_dev, uint8_t *rgb_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GBFUSION_H */
