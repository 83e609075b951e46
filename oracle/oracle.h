/*
 * oracle.h -- CPU restatement of the reference's dense-fusion hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU baseline leg may load it.  The
 * product path (libgbfusion) never calls it and has no CPU fallback.
 *
 * Every function restates a reference kernel body (paths relative to the
 * reference project, cited at each function in oracle_impl.h) in the
 * reference's operation order, in two precisions:
 *   *_f32  float arithmetic exactly as written (compiled -ffp-contract=off), with
 *          the voxel storage semantics of the chosen layout: the bit-exact
 *          parity target of the CUDA kernels for integer / byte results;
 *   *_f64  double arithmetic and unquantised voxel storage: the error
 *          reference (TSDF max-abs, raycast depth RMS, pose drift).
 *
 * Parity pins: the marching-cubes tables, computeHash and the coordinate
 * converters are checked against outputs of the reference's own source
 * compiled here (tests/golden/make_golden.py); the integration, z-range,
 * raycast, ICP-row and photometric-row bodies against outputs of the
 * reference's own kernels, compiled from its sources and run on a GPU
 * (tests/golden/make_kernel_golden.py, tests/test_ref_kernel_pins.py).  The kernels' third-party
 * steps (OpenCV bilateral / resize / pyrDown / cvtColor, Sophus SE(3), Eigen
 * LDLT) have no reference implementation available and are restated from
 * their documented definitions: parity of those steps is unpinned.
 */
#ifndef GBF_ORACLE_H
#define GBF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAX_LEVELS 5

typedef struct or_config {
    float voxel_size, truncation;
    float zmin_update, zmax_update, zmin_raycast, zmax_raycast;
    int32_t num_blocks;       /* pool size (blocks past it are not allocated) */
    int32_t voxel_layout;     /* 0 REF (int16 + f32 weight), 1 HALF (fp16 sdf + fp16 weight),
                                 2 SNORM (int16 rounded to nearest + fp16 weight) */
    int32_t num_levels;
    int32_t max_iterations[OR_MAX_LEVELS];
    float w_icp, w_rgb, icp_dist_thresh, icp_angle_thresh;
    int32_t bilateral;
    int32_t motion_prior;     /* 1: track from the last frame's motion (constant velocity) */
    int32_t threads;          /* OpenMP threads, 0 = default */
} or_config;

typedef struct or_intrinsics {
    int32_t width, height;
    float fx, fy, cx, cy;
} or_intrinsics;

typedef struct or_track_result {
    int32_t success, iterations;
    float icp_error, rgb_error, icp_inliers, rgb_inliers;
    double update[16];
} or_track_result;

typedef struct or_map_f32 or_map_f32;
typedef struct or_map_f64 or_map_f64;
typedef struct or_frame_f32 or_frame_f32;
typedef struct or_frame_f64 or_frame_f64;
typedef struct or_system_f32 or_system_f32;
typedef struct or_system_f64 or_system_f64;

#define OR_DECLARE(S)                                                                                              \
    or_map_##S *or_map_create_##S(const or_config *cfg, const or_intrinsics *K);                                   \
    void or_map_destroy_##S(or_map_##S *m);                                                                        \
    /* DenseMapping::update: alloc + visible + integrate; nmap (float4) NULL = 1/d^2 colour update */              \
    int or_fuse_##S(or_map_##S *m, const float *depth, const uint8_t *rgb, const float *nmap, const double T[16]); \
    /* DenseMapping::raycast: z-range tiles of the last fuse's visible blocks + march; vmap float4 */              \
    int or_raycast_##S(or_map_##S *m, const double T[16], float *vmap);                                            \
    /* the same, plus the hit's nearest voxel colour (3 bytes per pixel, white elsewhere) */                     \
    int or_raycast_maps_##S(or_map_##S *m, const double T[16], float *vmap, uint8_t *rgb);                        \
    /* DenseMapping::raycast_check_visibility: visible list recomputed for T, then raycast */                      \
    int or_raycast_check_visibility_##S(or_map_##S *m, const double T[16], float *vmap);                           \
    int64_t or_map_blocks_##S(const or_map_##S *m);                                                                \
    void or_ray_stats_##S(or_map_##S *m, const double T[16], long long out[7], int32_t *steps_per_pixel);            \
    int64_t or_map_export_##S(const or_map_##S *m, int32_t *coords, float *sdf, float *w, uint8_t *rgb,           \
                              int64_t max_blocks);                                                                 \
    int64_t or_visible_##S(const or_map_##S *m, int32_t *coords, int64_t max_blocks);                              \
    void or_zrange_##S(const or_map_##S *m, float *out);                                                           \
    int32_t or_render_blocks_##S(const or_map_##S *m);                                                             \
    /* marching cubes over all blocks; returns the triangle count (clamped writes) */                             \
    int64_t or_mesh_##S(const or_map_##S *m, int mode, float *vtx, void *attr, int64_t max_tris);                  \
    or_frame_##S *or_frame_create_##S(const or_config *cfg, const or_intrinsics *K);                               \
    void or_frame_destroy_##S(or_frame_##S *f);                                                                    \
    /* DeviceImage::upload: depth (metres) + rgb8 -> pyramids */                                                   \
    void or_build_pyramid_##S(or_frame_##S *f, const float *depth, const uint8_t *rgb);                           \
    /* copy one image: kind 0 vmap 1 nmap (float4) 2 intensity 3 dx 4 dy 5 depth */                                \
    void or_frame_get_##S(const or_frame_##S *f, int kind, int level, float *out);                                 \
    void or_frame_set_vmap_##S(or_frame_##S *f, const float *vmap0);                                               \
    /* icp_reduce + rgb_step sums for pose T (row-major 3x4 floats) */                                             \
    void or_reduce_##S(const or_frame_##S *ref, const or_frame_##S *cur, int level, const float T[12],            \
                       float stddev, double out[58]);                                                              \
    /* the same sums' terms per pixel, rounded to float: terms[p*58 + k] (0 without a correspondence) */          \
    void or_reduce_terms_##S(const or_frame_##S *ref, const or_frame_##S *cur, int level, const float T[12],      \
                             float stddev, float *terms);                                                          \
    /* DenseTracking::compute_transform */                                                                         \
    void or_track_##S(const or_frame_##S *ref, const or_frame_##S *cur, const double init[16],                    \
                      or_track_result *res);                                                                       \
    /* System::process_images */                                                                                   \
    or_system_##S *or_system_create_##S(const or_config *cfg, const or_intrinsics *K);                             \
    void or_system_destroy_##S(or_system_##S *s);                                                                  \
    void or_system_set_pose_##S(or_system_##S *s, const double T[16]);                                             \
    void or_system_get_pose_##S(const or_system_##S *s, double T[16]);                                             \
    void or_process_frame_##S(or_system_##S *s, const uint16_t *depth_mm, const uint8_t *rgb);                     \
    or_map_##S *or_system_map_##S(or_system_##S *s);                                                               \
    or_frame_##S *or_system_ref_##S(or_system_##S *s);                                                             \
    void or_system_last_result_##S(const or_system_##S *s, or_track_result *r);

OR_DECLARE(f32)
OR_DECLARE(f64)

/* shared integer helpers (reference map_struct.cu:143-148, 615-673) */
int or_compute_hash(int x, int y, int z, int n);
int or_floor_ref(float v);
void or_voxel_to_block(const int v[3], int out[3]);
void or_voxel_to_local(const int v[3], int out[3]);
int or_local_idx(const int l[3]);
int or_tri_table(int cube, int out[16]);   /* fills -1-terminated list, returns count */
/* renderScene / renderSceneTextured (cuda_imgproc.cu:17-108): float4 camera-frame
 * vertex / normal maps, rgb8 (NULL = untextured) -> rgba8 */
void or_render_scene(const float *vmap, const float *nmap, const uint8_t *rgb, int w, int h, uint8_t *out);
/* Column sums of an n x width float matrix, sequentially down each column in
 * float: plain (kahan = 0) or compensated (Kahan 1965, kahan = 1). */
void or_sum_f32(const float *terms, long long n, int width, int kahan, double *out);
/* sinf / expf of the FP32 oracle, from an installed table of device values or libm */
float or_sinf(float x);
float or_expf(float x);
float or_powf20(float x);
void or_trans_record(int enable);
long long or_trans_recorded(int kind, uint32_t *out, long long cap);
void or_trans_table(int kind, const uint32_t *x, const float *y, long long n);
long long or_trans_misses(int kind);
int or_edge_table(int cube);
short or_pack_sdf(float v);
float or_unpack_sdf(short v);

#ifdef __cplusplus
}
#endif
#endif
