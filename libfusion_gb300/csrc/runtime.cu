// runtime.cu -- host runtime behind the C ABI: sessions (one device arena
// each), the per-frame launch sequence, batches of sessions replayed from CUDA
// graphs, map export / import, and status reporting.
//
// The reference's host classes (DenseMapping, src/voxel_hashing/voxel_hashing.cpp;
// DenseOdometry / DenseTracking, src/tracking/rgbd_odometry.cpp and
// icp_tracker.cpp) allocate per call, read counts back to the host and run the
// Gauss-Newton loop on the CPU.  Here every frame is a fixed sequence of
// launches with device-resident counts and poses, so it can be captured once
// and replayed for many sessions.
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "gbf_device.cuh"
#include "gbf_internal.h"

namespace gbf {

namespace {
thread_local std::string g_last_error;
}

gbf_status set_error(gbf_status st, const char *msg) {
    g_last_error = msg ? msg : "";
    return st;
}

gbf_status cuda_error(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return GBF_OK;
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    g_last_error = m;
    if (e == cudaErrorMemoryAllocation) return GBF_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GBF_ERR_NO_DEVICE;
    return GBF_ERR_CUDA;
}

gbf_status check_cuda(const char *where) { return cuda_error(cudaGetLastError(), where); }

int reduce_ctas(int pixels) {
    const int per = kReduceThreads * kReducePixelsPerThread;
    return std::max(1, (pixels + per - 1) / per);
}

int reduce_tile(int level) { return level == 0 ? kReduceThreads * kReducePixelsPerThread : kCoarseReduceTile; }

gbf_status validate(const gbf_config *c, const gbf_intrinsics *K) {
    if (!c || !K) return set_error(GBF_ERR_INVALID_ARG, "null config or intrinsics");
    if (c->num_levels < 1 || c->num_levels > GBF_MAX_LEVELS)
        return set_error(GBF_ERR_INVALID_ARG, "num_levels must be in 1..5");
    const int div = 1 << (c->num_levels - 1);
    if (K->width < 64 || K->height < 64 || K->width % 8 || K->height % 8 || K->width % (2 * div) ||
        K->height % (2 * div) || (K->width / div) < 16 || (K->height / div) < 16)
        return set_error(GBF_ERR_INVALID_ARG,
                         "width/height must be multiples of 8 and of 2^num_levels, >= 64, coarsest level >= 16");
    if ((long long)K->width * K->height > (1 << 26)) return set_error(GBF_ERR_INVALID_ARG, "image too large");
    if (!(K->fx > 0) || !(K->fy > 0)) return set_error(GBF_ERR_INVALID_ARG, "focal lengths must be positive");
    if (!(c->voxel_size > 0) || !(c->truncation > 0)) return set_error(GBF_ERR_INVALID_ARG, "voxel/truncation must be > 0");
    if (c->num_buckets < 1 || c->num_blocks < 1) return set_error(GBF_ERR_INVALID_ARG, "table / pool size must be >= 1");
    if ((long long)c->num_blocks * kBlockVoxels > (1ll << 31) - 1)
        return set_error(GBF_ERR_INVALID_ARG, "num_blocks too large (voxel index must fit int32)");
    if (c->voxel_layout < 0 || c->voxel_layout >= kNumLayouts)
        return set_error(GBF_ERR_INVALID_ARG, "unknown voxel layout");
    if (c->max_probe < 1) return set_error(GBF_ERR_INVALID_ARG, "max_probe must be >= 1");
    if (c->motion_prior != 0 && c->motion_prior != 1) return set_error(GBF_ERR_INVALID_ARG, "motion_prior must be 0 or 1");
    for (int l = 0; l < c->num_levels; ++l)
        if (c->max_iterations[l] < 0 || c->max_iterations[l] > 1000)
            return set_error(GBF_ERR_INVALID_ARG, "max_iterations out of range");
    if (!(c->zmin_update < c->zmax_update) || !(c->zmin_raycast < c->zmax_raycast) || !(c->zmin_raycast > 0))
        return set_error(GBF_ERR_INVALID_ARG, "bad depth ranges");
    return GBF_OK;
}

ArenaLayout plan_arena(const gbf_config &c, const gbf_intrinsics &K) {
    ArenaLayout a;
    memset(&a, 0, sizeof(a));
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~size_t(255);
        return o;
    };
    const size_t pool = (size_t)c.num_blocks, nv = pool * kBlockVoxels;
    a.table = take((size_t)c.num_buckets * sizeof(HashSlot));
    a.bcoord = take(pool * sizeof(int4));
    a.bstamp = take(pool * sizeof(int));
    a.bfresh = take(pool);
    a.vis = take(pool * sizeof(int));
    a.mesh_off = take((pool + 1) * sizeof(int));
    a.vox_sw = take(nv * (c.voxel_layout == GBF_VOXEL_REF ? 8 : 4));
    a.vox_rgb = take(nv * 4);
    a.ctr = take(C_COUNT * sizeof(int));
    a.ts = take(sizeof(TrackState));
    const size_t P = (size_t)K.width * K.height;
    a.in_depth = take(P * 2);
    a.in_rgb = take(P * 3);
    a.depth_raw = take(P * 4);
    a.rgb4 = take(P * 4);
    a.nmap_ext = take(P * 16);
    a.fuse_px = take(P * 8);
    size_t w = K.width, h = K.height;
    for (int l = 0; l < c.num_levels; ++l) {
        const size_t p = w * h;
        a.depth[l] = take(p * 4);
        a.gx[l] = take(p * 4);
        a.gy[l] = take(p * 4);
        for (int s = 0; s < 2; ++s) {
            a.inten[s][l] = take(p * 4);
            a.vmap[s][l] = take(p * 16);
            a.nmap[s][l] = take(p * 16);
            a.igd[s][l] = take(p * 16);
        }
        w /= 2;
        h /= 2;
    }
    a.zr_min = take((size_t)(K.width / 8) * (K.height / 8) * 4);
    a.zr_max = take((size_t)(K.width / 8) * (K.height / 8) * 4);
    int max_ctas = 1;
    for (int l = 0, lw = K.width, lh = K.height; l < c.num_levels; ++l, lw /= 2, lh /= 2)
        max_ctas = std::max(max_ctas, (lw * lh + reduce_tile(l) - 1) / reduce_tile(l));
    a.partials = take((size_t)max_ctas * kPartialStride * 4);
    a.total = off;
    return a;
}

namespace {

__global__ void reset_table_kernel(HashSlot *t, int cap) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        HashSlot s;
        s.key = kEmptyKey;
        s.ptr = -1;
        s.pad = 0;
        t[i] = s;
    }
}

// canonical export of blocks [first, first+count): coords, float sdf/weight, rgb
template <int LAYOUT>
__global__ void export_kernel(const SessionView *__restrict__ svs, int first, int count, int *coords, float *sdf, float *w,
                              unsigned char *rgb) {
    const SessionView &sv = svs[0];
    for (int b = blockIdx.x; b < count; b += gridDim.x) {
        const int id = first + b;
        if (threadIdx.x == 0) {
            const int4 c = sv.bcoord[id];
            coords[b * 3 + 0] = c.x;
            coords[b * 3 + 1] = c.y;
            coords[b * 3 + 2] = c.z;
        }
        for (int i = threadIdx.x; i < kBlockVoxels; i += blockDim.x) {
            const Vox v = load_vox<LAYOUT>(sv, (size_t)id * kBlockVoxels + i);
            const size_t o = (size_t)b * kBlockVoxels + i;
            sdf[o] = v.sdf;
            w[o] = v.w;
            rgb[o * 3 + 0] = v.rgb.x;
            rgb[o * 3 + 1] = v.rgb.y;
            rgb[o * 3 + 2] = v.rgb.z;
        }
    }
}

template <int LAYOUT>
__global__ void import_kernel(const SessionView *__restrict__ svs, int count, const int *coords, const float *sdf, const float *w,
                              const unsigned char *rgb) {
    const SessionView &sv = svs[0];
    __shared__ int id_s;
    for (int b = blockIdx.x; b < count; b += gridDim.x) {
        if (threadIdx.x == 0) {
            const int x = coords[b * 3], y = coords[b * 3 + 1], z = coords[b * 3 + 2];
            id_s = coord_ok(x, y, z) ? insert_block(sv, pack_key(x, y, z), x, y, z, sv.ctr[C_FRAME]) : -1;
            if (id_s < 0 && !coord_ok(x, y, z)) raise_flag(sv, GBF_FLAG_COORD_RANGE);
        }
        __syncthreads();
        const int id = id_s;
        if (id >= 0) {
            for (int i = threadIdx.x; i < kBlockVoxels; i += blockDim.x) {
                const size_t o = (size_t)b * kBlockVoxels + i, vi = (size_t)id * kBlockVoxels + i;
                store_sw<LAYOUT>(sv, vi, sdf[o], w[o]);
                sv.vox_rgb[vi] = make_uchar4(rgb[o * 3], rgb[o * 3 + 1], rgb[o * 3 + 2], 0);
            }
            if (threadIdx.x == 0) sv.bfresh[id] = 0;
        }
        __syncthreads();
    }
}

void fill_levels(const gbf_config &c, const gbf_intrinsics &K, SessionView &v) {
    // IntrinsicMatrix + pyr_down (include/data_struct/intrinsic_matrix.h:27-37)
    float fx = K.fx, fy = K.fy, cx = K.cx, cy = K.cy;
    int w = K.width, h = K.height;
    for (int l = 0; l < c.num_levels; ++l) {
        LevelK &L = v.lv[l];
        L.w = w; L.h = h;
        L.fx = fx; L.fy = fy; L.cx = cx; L.cy = cy;
        L.invfx = 1.0f / fx;
        L.invfy = 1.0f / fy;
        v.red_tile[l] = reduce_tile(l);
        v.red_ctas[l] = std::max(1, (w * h + v.red_tile[l] - 1) / v.red_tile[l]);
        v.max_iter[l] = c.max_iterations[l];
        const float s = 0.5f;
        w = (int)(s * (float)w); h = (int)(s * (float)h);
        fx = s * fx; fy = s * fy; cx = s * cx; cy = s * cy;
    }
}

TrackState initial_track_state() {
    TrackState t;
    memset(&t, 0, sizeof(t));
    for (int i = 0; i < 12; ++i) {
        const double v = (i == 0 || i == 5 || i == 10) ? 1.0 : 0.0;
        t.pose[i] = t.map_pose[i] = t.est[i] = t.est_prev[i] = t.init[i] = t.update[i] = v;
    }
    t.icp_error = t.rgb_error = FLT_MAX;
    for (int i = 0; i < 12; ++i) t.map_twc[i] = t.map_tcw[i] = (float)t.map_pose[i];
    return t;
}

gbf_status reset_session(gbf_session *s, cudaStream_t st, bool keep_track = false) {
    reset_table_kernel<<<512, 256, 0, st>>>(s->view.table, s->cfg.num_buckets);
    cudaError_t e = cudaMemsetAsync(s->view.ctr, 0, C_COUNT * sizeof(int), st);
    if (e != cudaSuccess) return cuda_error(e, "reset");
    e = cudaMemsetAsync(s->view.bfresh, 0, (size_t)s->cfg.num_blocks, st);
    if (e != cudaSuccess) return cuda_error(e, "reset");
    if (!keep_track) {
        const TrackState t = initial_track_state();
        e = cudaMemcpyAsync(s->view.ts, &t, sizeof(t), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_error(e, "reset");
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "reset");
    return check_cuda("reset");
}

void to34(const double T[16], double o[12]) {
    for (int i = 0; i < 12; ++i) o[i] = T[i];
}
void to44(const double o[12], double T[16]) {
    for (int i = 0; i < 12; ++i) T[i] = o[i];
    T[12] = T[13] = T[14] = 0.0;
    T[15] = 1.0;
}

__global__ void map_pose_kernel(TrackState *ts) { update_map_floats(ts); }

gbf_status set_map_pose(gbf_session *s, const double T[16], cudaStream_t st) {
    double p[12];
    to34(T, p);
    // pageable source: the copy is staged before the call returns
    cudaError_t e = cudaMemcpyAsync(s->view.ts->map_pose, p, sizeof(p), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "set pose");
    map_pose_kernel<<<1, 1, 0, st>>>(s->view.ts);
    return check_cuda("set pose");
}

// One frame for `nslots` slots.  With `ev` (kPhases + 1 events) the phase
// boundaries are recorded: ingest, track, alloc+visible, integrate, z-range,
// march, post.
constexpr int kPhases = 7;
// Event marks at the phase boundaries (inside a capture an event record must
// become an event-record node of the graph).
struct PhaseMarks {
    cudaEvent_t *ev;
    bool capturing;
    PhaseMarks(cudaEvent_t *e, cudaStream_t st) : ev(e), capturing(false) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (ev) cudaStreamIsCapturing(st, &cs);
        capturing = cs == cudaStreamCaptureStatusActive;
    }
    void operator()(int i, cudaStream_t st) const {
        if (!ev) return;
        if (capturing) cudaEventRecordWithFlags(ev[i], st, cudaEventRecordExternal);
        else cudaEventRecord(ev[i], st);
    }
};

// First half of a frame: ingest and tracking (the pose of the frame is final
// after it).
void enqueue_first_half(const SessionView *d_sv, int nslots, const Extent &ex, const IngestArgs &in, cudaStream_t st,
                        cudaEvent_t *ev = nullptr) {
    PhaseMarks mark(ev, st);
    mark(0, st);
    launch_ingest(d_sv, nslots, ex, in, st);
    mark(1, st);
    launch_track(d_sv, nslots, ex, 1, st);
    mark(2, st);
}

// Second half: allocation, visibility, integration and the raycast that makes
// the next frame's reference maps.
void enqueue_second_half(const SessionView *d_sv, int nslots, const Extent &ex, const int *layouts, cudaStream_t st,
                         cudaEvent_t *ev = nullptr) {
    PhaseMarks mark(ev, st);
    launch_alloc_visible(d_sv, nslots, ex, st);
    mark(3, st);
    launch_integrate(d_sv, nslots, ex, 1, layouts, st);
    mark(4, st);
    launch_zrange(d_sv, nslots, ex, st);
    mark(5, st);
    launch_march(d_sv, nslots, ex, nullptr, 0, layouts, st);
    mark(6, st);
    launch_post(d_sv, nslots, ex, st);
    mark(7, st);
}

void enqueue_frame(const SessionView *d_sv, int nslots, const Extent &ex, const int *layouts, const IngestArgs &in,
                   cudaStream_t st, cudaEvent_t *ev = nullptr) {
    enqueue_first_half(d_sv, nslots, ex, in, st, ev);
    enqueue_second_half(d_sv, nslots, ex, layouts, st, ev);
}

// kernels launched by enqueue_frame
int kernels_per_frame(const Extent &ex, const int *layouts, int nslots) {
    int nl = 0;
    for (int l = 0; l < kNumLayouts; ++l) nl += layouts[l];
    return (1 + (ex.levels - 1) + 1) + track_launches(nslots, ex) + 3 + nl + 2 + nl + post_launches(ex);
}

}  // namespace

gbf_status reset_map(gbf_session *s) { return reset_session(s, nullptr, true); }

}  // namespace gbf

using namespace gbf;

extern "C" {

GBF_API const char *gbf_version(void) { return "libgbfusion 0.1.0 (sm_103a)"; }

GBF_API const char *gbf_last_error(void) { return g_last_error.c_str(); }

GBF_API gbf_status gbf_config_default(gbf_config *c) {
    if (!c) return set_error(GBF_ERR_INVALID_ARG, "gbf_config_default: null");
    memset(c, 0, sizeof(*c));
    // MapStruct<Device>::MapStruct (src/data_struct/map_struct.cu:17-35)
    c->voxel_size = 0.01f;
    c->truncation = 5.0f * c->voxel_size;  // MapState::truncation_dist (map_struct.cu:120-123)
    c->zmin_update = 0.3f;
    c->zmax_update = 1.5f;
    c->zmin_raycast = 0.3f;
    c->zmax_raycast = 1.5f;
    c->num_buckets = 200000;
    c->num_blocks = 200000;
    c->voxel_layout = GBF_VOXEL_REF;
    c->num_levels = 3;
    c->max_iterations[0] = 10;  // rgbd_odometry.cpp:33 (first three levels)
    c->max_iterations[1] = 5;
    c->max_iterations[2] = 3;
    c->max_iterations[3] = 3;
    c->max_iterations[4] = 3;
    c->w_icp = 1e6f;  // icp_tracker.cpp:89-90
    c->w_rgb = 1.0f;
    c->icp_dist_thresh = (float)0.01;                  // pose_estimator.cu:293
    c->icp_angle_thresh = (float)cos(30 * 3.14 / 180); // pose_estimator.cu:292
    c->bilateral = 1;
    c->max_probe = 64;
    return GBF_OK;
}

GBF_API gbf_status gbf_session_bytes(const gbf_config *cfg, const gbf_intrinsics *K, uint64_t *bytes) {
    gbf_status st = validate(cfg, K);
    if (st != GBF_OK) return st;
    if (!bytes) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_bytes: null");
    *bytes = plan_arena(*cfg, *K).total + sizeof(SessionView);
    return GBF_OK;
}

GBF_API gbf_status gbf_session_create(const gbf_config *cfg, const gbf_intrinsics *K, gbf_session **out) {
    if (!out) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_create: null out");
    *out = nullptr;
    gbf_status st = validate(cfg, K);
    if (st != GBF_OK) return st;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(GBF_ERR_NO_DEVICE, "gbf_session_create: no CUDA device");
    }
    gbf_session *s = new (std::nothrow) gbf_session();
    if (!s) return set_error(GBF_ERR_OUT_OF_MEMORY, "gbf_session_create: host allocation");
    s->cfg = *cfg;
    s->K = *K;
    cudaGetDevice(&s->device);
    s->lay = plan_arena(*cfg, *K);
    e = cudaMalloc(&s->arena, s->lay.total);
    if (e != cudaSuccess) {
        delete s;
        return cuda_error(e, "gbf_session_create: arena");
    }
    e = cudaMalloc(&s->d_view, sizeof(SessionView));
    if (e != cudaSuccess) {
        cudaFree(s->arena);
        delete s;
        return cuda_error(e, "gbf_session_create: view");
    }
    char *base = static_cast<char *>(s->arena);
    const ArenaLayout &a = s->lay;
    SessionView &v = s->view;
    memset(&v, 0, sizeof(v));
    v.active = 1;
    v.layout = cfg->voxel_layout;
    v.cap = cfg->num_buckets;
    v.cap_mask = (cfg->num_buckets & (cfg->num_buckets - 1)) == 0 ? cfg->num_buckets - 1 : -1;
    v.pool = cfg->num_blocks;
    v.max_probe = cfg->max_probe;
    v.motion_prior = cfg->motion_prior;
    v.voxel = cfg->voxel_size;
    v.inv_voxel = 1.0f / cfg->voxel_size;                         // MapState::inverse_voxel_size
    v.tau = cfg->truncation;
    v.inv_tau = (float)(1.0 / (double)cfg->truncation);           // depth_fusion.cu:377 (double division)
    v.step_scale = cfg->truncation * v.inv_voxel;                 // MapState::raycast_step_scale
    v.zmin_u = cfg->zmin_update;
    v.zmax_u = cfg->zmax_update;
    v.zmin_r = cfg->zmin_raycast;
    v.zmax_r = cfg->zmax_raycast;
    v.block_metric = (float)kBlockSide * cfg->voxel_size;        // MapState::block_size_metric
    v.w_icp = cfg->w_icp;
    v.w_rgb = cfg->w_rgb;
    v.icp_dist = cfg->icp_dist_thresh;
    v.icp_angle = cfg->icp_angle_thresh;
    v.bilateral = cfg->bilateral;
    v.levels = cfg->num_levels;
    fill_levels(*cfg, *K, v);
    v.table = reinterpret_cast<HashSlot *>(base + a.table);
    v.bcoord = reinterpret_cast<int4 *>(base + a.bcoord);
    v.bstamp = reinterpret_cast<int *>(base + a.bstamp);
    v.bfresh = reinterpret_cast<unsigned char *>(base + a.bfresh);
    v.vis = reinterpret_cast<int *>(base + a.vis);
    v.mesh_off = reinterpret_cast<int *>(base + a.mesh_off);
    v.vox_sw = base + a.vox_sw;
    v.vox_rgb = reinterpret_cast<uchar4 *>(base + a.vox_rgb);
    v.ctr = reinterpret_cast<int *>(base + a.ctr);
    v.ts = reinterpret_cast<TrackState *>(base + a.ts);
    v.in_depth = reinterpret_cast<uint16_t *>(base + a.in_depth);
    v.in_rgb = reinterpret_cast<uint8_t *>(base + a.in_rgb);
    v.depth_raw = reinterpret_cast<float *>(base + a.depth_raw);
    v.rgb4 = reinterpret_cast<uchar4 *>(base + a.rgb4);
    v.nmap_ext = reinterpret_cast<float4 *>(base + a.nmap_ext);
    v.fuse_px = reinterpret_cast<float2 *>(base + a.fuse_px);
    for (int l = 0; l < cfg->num_levels; ++l) {
        v.depth[l] = reinterpret_cast<float *>(base + a.depth[l]);
        v.gx[l] = reinterpret_cast<float *>(base + a.gx[l]);
        v.gy[l] = reinterpret_cast<float *>(base + a.gy[l]);
        for (int k = 0; k < 2; ++k) {
            v.inten[k][l] = reinterpret_cast<float *>(base + a.inten[k][l]);
            v.vmap[k][l] = reinterpret_cast<float4 *>(base + a.vmap[k][l]);
            v.nmap[k][l] = reinterpret_cast<float4 *>(base + a.nmap[k][l]);
            v.igd[k][l] = reinterpret_cast<float4 *>(base + a.igd[k][l]);
        }
    }
    v.zr_min = reinterpret_cast<float *>(base + a.zr_min);
    v.zr_max = reinterpret_cast<float *>(base + a.zr_max);
    v.zr_w = K->width / 8;
    v.zr_h = K->height / 8;
    v.partials = reinterpret_cast<float *>(base + a.partials);

    Extent &ex = s->ex;
    memset(&ex, 0, sizeof(ex));
    ex.w = K->width;
    ex.h = K->height;
    ex.max_pool = cfg->num_blocks;
    ex.levels = cfg->num_levels;
    for (int l = 0; l < cfg->num_levels; ++l) {
        ex.max_red[l] = v.red_ctas[l];
        ex.max_iter[l] = cfg->max_iterations[l];
    }
    s->layouts[cfg->voxel_layout] = 1;

    e = cudaMemcpy(s->d_view, &v, sizeof(v), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        gbf_session_destroy(s);
        return cuda_error(e, "gbf_session_create: upload view");
    }
    st = reset_session(s, 0);
    if (st != GBF_OK) {
        gbf_session_destroy(s);
        return st;
    }
    *out = s;
    return GBF_OK;
}

GBF_API gbf_status gbf_session_destroy(gbf_session *s) {
    if (!s) return GBF_OK;
    cudaDeviceSynchronize();
    if (s->d_view) cudaFree(s->d_view);
    if (s->arena) cudaFree(s->arena);
    delete s;
    return check_cuda("gbf_session_destroy");
}

GBF_API gbf_status gbf_session_reset(gbf_session *s, void *stream) {
    if (!s) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_reset: null");
    return reset_session(s, (cudaStream_t)stream);
}

GBF_API gbf_status gbf_session_inputs(gbf_session *s, uint16_t **depth, uint8_t **rgb) {
    if (!s || !depth || !rgb) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_inputs: null");
    *depth = s->view.in_depth;
    *rgb = s->view.in_rgb;
    return GBF_OK;
}

// Rows of an image into dense rows: one contiguous copy when the source rows
// are dense too (a camera frame usually is).  A pitched copy from pinned host
// memory measured 0.43 ms slower per 64-frame tick of the batch it overlapped
// (64 x 640x480 depth + colour staged per tick).
static cudaError_t copy_rows(void *dst, const void *src, int64_t src_pitch, size_t row_bytes, int rows,
                             cudaStream_t st) {
    if (src_pitch == (int64_t)row_bytes)
        return cudaMemcpyAsync(dst, src, row_bytes * (size_t)rows, cudaMemcpyDefault, st);
    return cudaMemcpy2DAsync(dst, row_bytes, src, (size_t)src_pitch, row_bytes, rows, cudaMemcpyDefault, st);
}

GBF_API gbf_status gbf_session_stage(gbf_session *s, const uint16_t *depth, int64_t depth_pitch, const uint8_t *rgb,
                                     int64_t rgb_pitch, void *stream) {
    if (!s || !depth || !rgb) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_stage: null");
    const int W = s->K.width, H = s->K.height;
    if (depth_pitch < W * 2 || rgb_pitch < W * 3)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_session_stage: pitch smaller than a row");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = copy_rows(s->view.in_depth, depth, depth_pitch, (size_t)W * 2, H, st);
    if (e == cudaSuccess) e = copy_rows(s->view.in_rgb, rgb, rgb_pitch, (size_t)W * 3, H, st);
    return cuda_error(e, "gbf_session_stage");
}

GBF_API gbf_status gbf_set_pose(gbf_session *s, const double T[16], void *stream) {
    if (!s || !T) return set_error(GBF_ERR_INVALID_ARG, "gbf_set_pose: null");
    double p[12];
    to34(T, p);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(s->view.ts->pose, p, sizeof(p), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->view.ts->map_pose, p, sizeof(p), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) map_pose_kernel<<<1, 1, 0, st>>>(s->view.ts);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_error(e, "gbf_set_pose");
}

GBF_API gbf_status gbf_get_pose(gbf_session *s, double T[16], void *stream) {
    if (!s || !T) return set_error(GBF_ERR_INVALID_ARG, "gbf_get_pose: null");
    double p[12];
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(p, s->view.ts->pose, sizeof(p), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_get_pose");
    to44(p, T);
    return GBF_OK;
}

static void fill_result(const TrackState &t, gbf_track_result *r) {
    r->success = t.success;
    r->iterations = t.iterations;
    r->icp_error = t.icp_error;
    r->rgb_error = t.rgb_error;
    r->icp_inliers = t.icp_inliers;
    r->rgb_inliers = t.rgb_inliers;
    to44(t.update, r->update);
}

GBF_API gbf_status gbf_get_stats(gbf_session *s, gbf_frame_stats *out, void *stream) {
    if (!s || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_get_stats: null");
    cudaStream_t st = (cudaStream_t)stream;
    int ctr[C_COUNT];
    TrackState t;
    cudaError_t e = cudaMemcpyAsync(ctr, s->view.ctr, sizeof(ctr), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&t, s->view.ts, sizeof(t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_get_stats");
    out->frame_index = t.frame_index;
    out->allocated_blocks = std::min(ctr[C_NUSED], s->cfg.num_blocks);
    out->visible_blocks = ctr[C_NVIS];
    out->render_blocks_valid = ctr[C_RENDER];
    out->status = (uint32_t)ctr[C_STATUS];
    fill_result(t, &out->track);
    for (int l = 0; l < GBF_MAX_LEVELS; ++l) out->level_iterations[l] = t.level_iters[l];
    out->pixel_iterations = t.pixel_iterations;
    out->integrated_blocks = t.integrated_blocks;
    return GBF_OK;
}

// A kernel reads or writes a caller's image as rows of `elem`-byte elements:
// its base address and its pitch must both be multiples of elem.
static bool rows_aligned(const void *p, int64_t pitch, int elem) {
    return reinterpret_cast<uintptr_t>(p) % elem == 0 && pitch % elem == 0;
}

GBF_API gbf_status gbf_fuse(gbf_session *s, const float *depth, int64_t depth_pitch, const uint8_t *rgb,
                            int64_t rgb_pitch, const float *nmap, int64_t nmap_pitch, const double T[16],
                            void *stream) {
    if (!s || !depth || !rgb || !T) return set_error(GBF_ERR_INVALID_ARG, "gbf_fuse: null");
    if (depth_pitch < s->K.width * 4 || rgb_pitch < s->K.width * 3 || (nmap && nmap_pitch < s->K.width * 16))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_fuse: pitch smaller than a row");
    if (!rows_aligned(depth, depth_pitch, 4) || (nmap && !rows_aligned(nmap, nmap_pitch, 16)))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_fuse: depth rows must be 4-byte and normal rows 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    gbf_status r = set_map_pose(s, T, st);
    if (r != GBF_OK) return r;
    FuseImport in{depth, depth_pitch, rgb, rgb_pitch, nmap, nmap_pitch};
    launch_fuse_import(s->d_view, s->ex, in, st);
    launch_fuse(s->d_view, 1, s->ex, nmap ? 2 : 0, s->layouts, st);
    return check_cuda("gbf_fuse");
}

GBF_API gbf_status gbf_raycast(gbf_session *s, const double T[16], float *vmap, int64_t vmap_pitch, void *stream) {
    if (!s || !T || !vmap) return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast: null");
    if (vmap_pitch < s->K.width * 16) return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast: pitch smaller than a row");
    if (!rows_aligned(vmap, vmap_pitch, 16))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast: vertex-map rows must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    gbf_status r = set_map_pose(s, T, st);
    if (r != GBF_OK) return r;
    launch_raycast(s->d_view, 1, s->ex, reinterpret_cast<float4 *>(vmap), vmap_pitch, 0, s->layouts, st);
    return check_cuda("gbf_raycast");
}

GBF_API gbf_status gbf_raycast_maps(gbf_session *s, const double T[16], float *vmap, int64_t vmap_pitch,
                                    float *nmap, int64_t nmap_pitch, uint8_t *rgb, int64_t rgb_pitch, void *stream) {
    if (!s || !T || !vmap) return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast_maps: null");
    const int W = s->K.width, H = s->K.height;
    if (vmap_pitch < W * 16LL || (nmap && nmap_pitch < W * 16LL) || (rgb && rgb_pitch < W * 3LL))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast_maps: pitch smaller than a row");
    if (!rows_aligned(vmap, vmap_pitch, 16) || (nmap && !rows_aligned(nmap, nmap_pitch, 16)))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast_maps: vertex and normal rows must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    gbf_status r = set_map_pose(s, T, st);
    if (r != GBF_OK) return r;
    launch_raycast(s->d_view, 1, s->ex, reinterpret_cast<float4 *>(vmap), vmap_pitch, 0, s->layouts, st, rgb,
                   rgb_pitch);
    if (nmap)
        launch_nmap_of(reinterpret_cast<const float4 *>(vmap), vmap_pitch, reinterpret_cast<float4 *>(nmap),
                       nmap_pitch, W, H, st);
    return check_cuda("gbf_raycast_maps");
}

GBF_API gbf_status gbf_raycast_check_visibility(gbf_session *s, const double T[16], float *vmap, int64_t vmap_pitch,
                                                void *stream) {
    if (!s || !T || !vmap) return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast_check_visibility: null");
    if (vmap_pitch < s->K.width * 16)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast_check_visibility: pitch smaller than a row");
    if (!rows_aligned(vmap, vmap_pitch, 16))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_raycast_check_visibility: vertex-map rows must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    gbf_status r = set_map_pose(s, T, st);
    if (r != GBF_OK) return r;
    launch_visible_frustum(s->d_view, 1, s->ex, st);
    launch_raycast(s->d_view, 1, s->ex, reinterpret_cast<float4 *>(vmap), vmap_pitch, 0, s->layouts, st);
    return check_cuda("gbf_raycast_check_visibility");
}

GBF_API gbf_status gbf_render_scene(const float *vmap, int64_t vmap_pitch, const float *nmap, int64_t nmap_pitch,
                                    const uint8_t *rgb, int64_t rgb_pitch, int32_t width, int32_t height,
                                    uint8_t *out, int64_t out_pitch, void *stream) {
    if (!vmap || !nmap || !out || width < 1 || height < 1)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_render_scene: null or empty");
    if (vmap_pitch < width * 16LL || nmap_pitch < width * 16LL || out_pitch < width * 4LL ||
        (rgb && rgb_pitch < width * 3LL))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_render_scene: pitch smaller than a row");
    if (!rows_aligned(vmap, vmap_pitch, 16) || !rows_aligned(nmap, nmap_pitch, 16) || !rows_aligned(out, out_pitch, 4))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_render_scene: map rows must be 16-byte and output rows 4-byte aligned");
    launch_render(reinterpret_cast<const float4 *>(vmap), vmap_pitch, reinterpret_cast<const float4 *>(nmap),
                  nmap_pitch, rgb, rgb_pitch, 3, width, height, reinterpret_cast<uchar4 *>(out), out_pitch,
                  (cudaStream_t)stream);
    return check_cuda("gbf_render_scene");
}

GBF_API gbf_status gbf_session_render(gbf_session *s, int32_t textured, uint8_t *out, int64_t out_pitch,
                                      void *stream) {
    if (!s || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_render: null");
    const int W = s->K.width, H = s->K.height;
    if (out_pitch < W * 4LL) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_render: pitch smaller than a row");
    if (!rows_aligned(out, out_pitch, 4))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_session_render: output rows must be 4-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    // the reference frame's maps: the model prediction of the last raycast
    int idx = 0;
    cudaError_t e = cudaMemcpyAsync(&idx, &s->view.ts->idx, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_render");
    launch_render(s->view.vmap[idx][0], W * 16LL, s->view.nmap[idx][0], W * 16LL,
                  textured ? reinterpret_cast<const uint8_t *>(s->view.rgb4) : nullptr, W * 4LL, 4, W, H,
                  reinterpret_cast<uchar4 *>(out), out_pitch, st);
    return check_cuda("gbf_session_render");
}

GBF_API gbf_status gbf_extract_mesh(gbf_session *s, int32_t mode, float *vtx, void *attr, uint64_t max_tris,
                                    uint64_t *n_tris, void *stream) {
    if (!s || !vtx || !n_tris) return set_error(GBF_ERR_INVALID_ARG, "gbf_extract_mesh: null");
    if (mode < GBF_MESH_VERTEX || mode > GBF_MESH_COLOUR) return set_error(GBF_ERR_INVALID_ARG, "bad mesh mode");
    if (mode != GBF_MESH_VERTEX && !attr) return set_error(GBF_ERR_INVALID_ARG, "gbf_extract_mesh: null attr");
    cudaStream_t st = (cudaStream_t)stream;
    const long long mt = (long long)std::min<uint64_t>(max_tris, (uint64_t)INT32_MAX);
    launch_mesh(s->d_view, s->ex, s->cfg.voxel_layout, mode, vtx, attr, mt, s->view.mesh_off, st);
    gbf_status r = check_cuda("gbf_extract_mesh");
    if (r != GBF_OK) return r;
    int total = 0;
    cudaError_t e = cudaMemcpyAsync(&total, s->view.ctr + C_MESH_TRIS, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_extract_mesh");
    *n_tris = std::min<uint64_t>((uint64_t)total, max_tris);
    return GBF_OK;
}

GBF_API gbf_status gbf_build_pyramid(gbf_session *s, int32_t which, const float *depth, int64_t depth_pitch,
                                     const uint8_t *rgb, int64_t rgb_pitch, void *stream) {
    if (!s || !depth || !rgb) return set_error(GBF_ERR_INVALID_ARG, "gbf_build_pyramid: null");
    if (which != 0 && which != 1) return set_error(GBF_ERR_INVALID_ARG, "gbf_build_pyramid: which must be 0 or 1");
    if (depth_pitch < s->K.width * 4 || rgb_pitch < s->K.width * 3)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_build_pyramid: pitch smaller than a row");
    if (!rows_aligned(depth, depth_pitch, 4))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_build_pyramid: depth rows must be 4-byte aligned");
    IngestArgs a{which, 2, depth, depth_pitch, rgb, rgb_pitch};
    launch_ingest(s->d_view, 1, s->ex, a, (cudaStream_t)stream);
    return check_cuda("gbf_build_pyramid");
}

GBF_API gbf_status gbf_reduce(gbf_session *s, int32_t level, const double T[16], float stddev, double out[58],
                              void *stream) {
    if (!s || !T || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_reduce: null");
    if (level < 0 || level >= s->cfg.num_levels) return set_error(GBF_ERR_INVALID_ARG, "gbf_reduce: bad level");
    cudaStream_t st = (cudaStream_t)stream;
    float p[12];
    for (int i = 0; i < 12; ++i) p[i] = (float)T[i];
    launch_reduce_once(s->d_view, s->ex, level, p, stddev, st);
    gbf_status r = check_cuda("gbf_reduce");
    if (r != GBF_OK) return r;
    cudaError_t e = cudaMemcpyAsync(out, s->view.ts->last_sums, sizeof(double) * kReduceWidth,
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_error(e, "gbf_reduce");
}

GBF_API gbf_status gbf_track(gbf_session *s, const double init[16], gbf_track_result *out, void *stream) {
    if (!s || !init || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_track: null");
    cudaStream_t st = (cudaStream_t)stream;
    double p[12];
    to34(init, p);
    cudaError_t e = cudaMemcpyAsync(s->view.ts->init, p, sizeof(p), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_track");
    launch_track(s->d_view, 1, s->ex, 0, st);
    gbf_status r = check_cuda("gbf_track");
    if (r != GBF_OK) return r;
    TrackState t;
    e = cudaMemcpyAsync(&t, s->view.ts, sizeof(t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_track");
    fill_result(t, out);
    return GBF_OK;
}

GBF_API gbf_status gbf_get_image(gbf_session *s, int32_t which, int32_t kind, int32_t level, void *out,
                                 int64_t pitch, void *stream) {
    if (!s || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_get_image: null");
    if (level < 0 || level >= s->cfg.num_levels || kind < 0 || kind > 5 || (which != 0 && which != 1))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_get_image: bad level/kind/which");
    cudaStream_t st = (cudaStream_t)stream;
    int idx = 0;
    cudaError_t e = cudaMemcpyAsync(&idx, &s->view.ts->idx, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_get_image");
    const int set = which ? idx : 1 - idx;
    const SessionView &v = s->view;
    const void *src = nullptr;
    size_t elem = 4;
    switch (kind) {
        case 0: src = v.vmap[set][level]; elem = 16; break;
        case 1: src = v.nmap[set][level]; elem = 16; break;
        case 2: src = v.inten[set][level]; break;
        case 3: src = v.gx[level]; break;
        case 4: src = v.gy[level]; break;
        default: src = v.depth[level]; break;
    }
    const int w = v.lv[level].w, h = v.lv[level].h;
    if (pitch < (int64_t)(w * elem)) return set_error(GBF_ERR_INVALID_ARG, "gbf_get_image: pitch smaller than a row");
    e = cudaMemcpy2DAsync(out, pitch, src, w * elem, w * elem, h, cudaMemcpyDefault, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_error(e, "gbf_get_image");
}

GBF_API gbf_status gbf_process_frame(gbf_session *s, const uint16_t *depth, int64_t depth_pitch, const uint8_t *rgb,
                                     int64_t rgb_pitch, void *stream) {
    if (!s || !depth || !rgb) return set_error(GBF_ERR_INVALID_ARG, "gbf_process_frame: null");
    if (depth_pitch < s->K.width * 2 || rgb_pitch < s->K.width * 3)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_process_frame: pitch smaller than a row");
    if (!rows_aligned(depth, depth_pitch, 2))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_process_frame: depth rows must be 2-byte aligned");
    IngestArgs a{0, 1, depth, depth_pitch, rgb, rgb_pitch};
    enqueue_frame(s->d_view, 1, s->ex, s->layouts, a, (cudaStream_t)stream);
    return check_cuda("gbf_process_frame");
}

GBF_API gbf_status gbf_process_frame_staged(gbf_session *s, void *stream) {
    if (!s) return set_error(GBF_ERR_INVALID_ARG, "gbf_process_frame_staged: null");
    IngestArgs a{0, 0, nullptr, 0, nullptr, 0};
    enqueue_frame(s->d_view, 1, s->ex, s->layouts, a, (cudaStream_t)stream);
    return check_cuda("gbf_process_frame_staged");
}

GBF_API gbf_status gbf_map_export(gbf_session *s, int32_t *coords, float *sdf, float *weight, uint8_t *rgb,
                                  int64_t max_blocks, int64_t *n_blocks) {
    if (!s || !n_blocks) return set_error(GBF_ERR_INVALID_ARG, "gbf_map_export: null");
    int used = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&used, s->view.ctr + C_NUSED, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "gbf_map_export");
    const int n = std::min(used, s->cfg.num_blocks);
    *n_blocks = n;
    if (!coords) return GBF_OK;  // size query
    if (!sdf || !weight || !rgb) return set_error(GBF_ERR_INVALID_ARG, "gbf_map_export: null output");
    if (max_blocks < n) return set_error(GBF_ERR_CAPACITY, "gbf_map_export: output holds fewer blocks than allocated");
    const int chunk = 4096;
    int *d_c = nullptr;
    float *d_s = nullptr, *d_w = nullptr;
    unsigned char *d_r = nullptr;
    e = cudaMalloc(&d_c, chunk * 3 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_s, (size_t)chunk * kBlockVoxels * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_w, (size_t)chunk * kBlockVoxels * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_r, (size_t)chunk * kBlockVoxels * 3);
    for (int first = 0; e == cudaSuccess && first < n; first += chunk) {
        const int cnt = std::min(chunk, n - first);
        if (s->cfg.voxel_layout == GBF_VOXEL_REF)
            export_kernel<GBF_VOXEL_REF><<<std::min(cnt, 1024), 256>>>(s->d_view, first, cnt, d_c, d_s, d_w, d_r);
        else if (s->cfg.voxel_layout == GBF_VOXEL_HALF)
            export_kernel<GBF_VOXEL_HALF><<<std::min(cnt, 1024), 256>>>(s->d_view, first, cnt, d_c, d_s, d_w, d_r);
        else
            export_kernel<GBF_VOXEL_SNORM><<<std::min(cnt, 1024), 256>>>(s->d_view, first, cnt, d_c, d_s, d_w, d_r);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(coords + (size_t)first * 3, d_c, (size_t)cnt * 3 * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(sdf + (size_t)first * kBlockVoxels, d_s, (size_t)cnt * kBlockVoxels * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(weight + (size_t)first * kBlockVoxels, d_w, (size_t)cnt * kBlockVoxels * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(rgb + (size_t)first * kBlockVoxels * 3, d_r, (size_t)cnt * kBlockVoxels * 3, cudaMemcpyDeviceToHost);
    }
    cudaFree(d_c);
    cudaFree(d_s);
    cudaFree(d_w);
    cudaFree(d_r);
    return cuda_error(e, "gbf_map_export");
}

GBF_API gbf_status gbf_map_import(gbf_session *s, const int32_t *coords, const float *sdf, const float *weight,
                                  const uint8_t *rgb, int64_t n_blocks) {
    if (!s || (n_blocks > 0 && (!coords || !sdf || !weight || !rgb)))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_map_import: null");
    const int chunk = 4096;
    int *d_c = nullptr;
    float *d_s = nullptr, *d_w = nullptr;
    unsigned char *d_r = nullptr;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMalloc(&d_c, chunk * 3 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_s, (size_t)chunk * kBlockVoxels * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_w, (size_t)chunk * kBlockVoxels * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_r, (size_t)chunk * kBlockVoxels * 3);
    for (int64_t first = 0; e == cudaSuccess && first < n_blocks; first += chunk) {
        const int cnt = (int)std::min<int64_t>(chunk, n_blocks - first);
        e = cudaMemcpy(d_c, coords + first * 3, (size_t)cnt * 3 * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_s, sdf + first * kBlockVoxels, (size_t)cnt * kBlockVoxels * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_w, weight + first * kBlockVoxels, (size_t)cnt * kBlockVoxels * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_r, rgb + first * kBlockVoxels * 3, (size_t)cnt * kBlockVoxels * 3, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) break;
        if (s->cfg.voxel_layout == GBF_VOXEL_REF)
            import_kernel<GBF_VOXEL_REF><<<std::min(cnt, 1024), 256>>>(s->d_view, cnt, d_c, d_s, d_w, d_r);
        else if (s->cfg.voxel_layout == GBF_VOXEL_HALF)
            import_kernel<GBF_VOXEL_HALF><<<std::min(cnt, 1024), 256>>>(s->d_view, cnt, d_c, d_s, d_w, d_r);
        else
            import_kernel<GBF_VOXEL_SNORM><<<std::min(cnt, 1024), 256>>>(s->d_view, cnt, d_c, d_s, d_w, d_r);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    cudaFree(d_c);
    cudaFree(d_s);
    cudaFree(d_w);
    cudaFree(d_r);
    return cuda_error(e, "gbf_map_import");
}

GBF_API gbf_status gbf_visible_blocks(gbf_session *s, int32_t *coords, int64_t max_blocks, int64_t *n_blocks) {
    if (!s || !n_blocks) return set_error(GBF_ERR_INVALID_ARG, "gbf_visible_blocks: null");
    int ctr[C_COUNT];
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(ctr, s->view.ctr, sizeof(ctr), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "gbf_visible_blocks");
    const int nv = ctr[C_NVIS], nu = std::min(ctr[C_NUSED], s->cfg.num_blocks);
    *n_blocks = nv;
    if (!coords) return GBF_OK;
    if (max_blocks < nv) return set_error(GBF_ERR_CAPACITY, "gbf_visible_blocks: output too small");
    std::vector<int> ids(nv);
    std::vector<int4> bc(nu);
    if (nv) e = cudaMemcpy(ids.data(), s->view.vis, nv * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nu) e = cudaMemcpy(bc.data(), s->view.bcoord, nu * sizeof(int4), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "gbf_visible_blocks");
    for (int i = 0; i < nv; ++i) {
        const int id = ids[i] & 0x7fffffff;
        if (id >= nu) return set_error(GBF_ERR_CUDA, "gbf_visible_blocks: corrupt visible list");
        coords[i * 3] = bc[id].x;
        coords[i * 3 + 1] = bc[id].y;
        coords[i * 3 + 2] = bc[id].z;
    }
    return GBF_OK;
}

GBF_API gbf_status gbf_zrange(gbf_session *s, float *out, int64_t max_cells) {
    if (!s || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_zrange: null");
    const int n = s->view.zr_w * s->view.zr_h;
    if (max_cells < n) return set_error(GBF_ERR_CAPACITY, "gbf_zrange: output too small");
    std::vector<float> a(n), b(n);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(a.data(), s->view.zr_min, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(b.data(), s->view.zr_max, n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "gbf_zrange");
    for (int i = 0; i < n; ++i) {
        out[2 * i] = a[i];
        out[2 * i + 1] = b[i];
    }
    return GBF_OK;
}

// ---- batches ------------------------------------------------------------------------

static gbf_status batch_flush(gbf_batch *b, cudaStream_t st);

GBF_API gbf_status gbf_batch_create(int32_t max_sessions, gbf_batch **out) {
    if (!out || max_sessions < 1 || max_sessions > 4096)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_create: 1..4096 sessions");
    *out = nullptr;
    gbf_batch *b = new (std::nothrow) gbf_batch();
    if (!b) return set_error(GBF_ERR_OUT_OF_MEMORY, "gbf_batch_create: host allocation");
    b->max_slots = max_sessions;
    b->sessions.assign(max_sessions, nullptr);
    b->in_depth.assign(max_sessions, nullptr);
    b->in_rgb.assign(max_sessions, nullptr);
    b->owed.assign(max_sessions, 0);
    const size_t bytes = sizeof(SessionView) * max_sessions;
    cudaError_t e = cudaMallocHost(&b->h_views[0], bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_views[1], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_views, bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_views_b[0], bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_views_b[1], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_views_b, bytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev[1], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
    for (int g = 0; e == cudaSuccess && g < gbf_batch::kMaxGroups - 1; ++g) {
        e = cudaStreamCreateWithFlags(&b->side[g], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[g], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int k = 0; k < 2; ++k) {
        b->stg_depth[k].assign(max_sessions, nullptr);
        b->stg_rgb[k].assign(max_sessions, nullptr);
        b->stg_pixels[k].assign(max_sessions, 0);
        b->staged[k].assign(max_sessions, 0);
        b->staged_ev[k].assign(max_sessions, nullptr);
        if (e == cudaSuccess) e = cudaMalloc(&b->d_res[k], sizeof(gbf_slot_result) * max_sessions);
        if (e == cudaSuccess) e = cudaMallocHost(&b->h_res[k], sizeof(gbf_slot_result) * max_sessions);
        if (e == cudaSuccess) memset(b->h_res[k], 0, sizeof(gbf_slot_result) * max_sessions);
    }
    if (e != cudaSuccess) {
        gbf_batch_destroy(b);
        return cuda_error(e, "gbf_batch_create");
    }
    for (int k = 0; k < 2; ++k) {
        memset(b->h_views[k], 0, bytes);
        memset(b->h_views_b[k], 0, bytes);
    }
    *out = b;
    return GBF_OK;
}

static void batch_invalidate(gbf_batch *b) {
    for (int k = 0; k < 2; ++k)
        if (b->exec[k]) {
            cudaGraphExecDestroy(b->exec[k]);
            b->exec[k] = nullptr;
        }
}

GBF_API gbf_status gbf_batch_destroy(gbf_batch *b) {
    if (!b) return GBF_OK;
    // The caller guarantees that no other gbf_batch_* call on b is pending or
    // starts once destroy begins; taking the lock only orders this thread
    // after a call that returned on another thread.
    std::unique_lock<std::mutex> lock(b->mu);
    if (b->d_views_b) batch_flush(b, nullptr);  // the sessions outlive the batch: fuse what is owed
    cudaDeviceSynchronize();
    batch_invalidate(b);
    for (int k = 0; k < 2; ++k) {
        if (b->h_views[k]) cudaFreeHost(b->h_views[k]);
        if (b->h_views_b[k]) cudaFreeHost(b->h_views_b[k]);
        if (b->ev[k]) cudaEventDestroy(b->ev[k]);
    }
    if (b->d_views) cudaFree(b->d_views);
    if (b->d_views_b) cudaFree(b->d_views_b);
    if (b->own) cudaStreamDestroy(b->own);
    for (int g = 0; g < gbf_batch::kMaxGroups - 1; ++g) {
        if (b->side[g]) cudaStreamDestroy(b->side[g]);
        if (b->join[g]) cudaEventDestroy(b->join[g]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    for (int k = 0; k < 2; ++k) {
        for (size_t i = 0; i < b->stg_depth[k].size(); ++i) {
            if (b->stg_depth[k][i]) cudaFree(b->stg_depth[k][i]);
            if (b->stg_rgb[k][i]) cudaFree(b->stg_rgb[k][i]);
            if (b->staged_ev[k][i]) cudaEventDestroy(b->staged_ev[k][i]);
        }
        if (b->d_res[k]) cudaFree(b->d_res[k]);
        if (b->h_res[k]) cudaFreeHost(b->h_res[k]);
    }
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 8; ++i)
            if (b->pev[k][i]) cudaEventDestroy(b->pev[k][i]);
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 2; ++i)
            if (b->tev[k][i]) cudaEventDestroy(b->tev[k][i]);
    lock.unlock();
    delete b;
    return check_cuda("gbf_batch_destroy");
}

static void batch_reshape(gbf_batch *b);

GBF_API gbf_status gbf_batch_set(gbf_batch *b, int32_t slot, gbf_session *s) {
    if (!b || slot < 0 || slot >= b->max_slots) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set: bad slot");
    std::lock_guard<std::mutex> lock(b->mu);
    gbf_status fs = batch_flush(b, nullptr);
    if (fs != GBF_OK) return fs;
    // a previous tick may still read the mirrors
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) cudaEventSynchronize(b->ev[k]);
    b->sessions[slot] = s;
    b->staged[0][slot] = b->staged[1][slot] = 0;
    batch_reshape(b);
    return GBF_OK;
}

// The tick's shape: the reserved floor, raised by the sessions in the slots.
static void batch_reshape(gbf_batch *b) {
    int nslots = b->floor_slots, layouts[kNumLayouts] = {};
    for (int i = 0; i < kNumLayouts; ++i) layouts[i] = b->floor_layouts[i];
    Extent ex = b->floor_ex;
    for (int i = 0; i < b->max_slots; ++i) {
        gbf_session *t = b->sessions[i];
        if (!t) continue;
        nslots = std::max(nslots, i + 1);
        ex.w = std::max(ex.w, t->ex.w);
        ex.h = std::max(ex.h, t->ex.h);
        ex.max_pool = std::max(ex.max_pool, t->ex.max_pool);
        ex.levels = std::max(ex.levels, t->ex.levels);
        for (int l = 0; l < kMaxLevels; ++l) {
            ex.max_red[l] = std::max(ex.max_red[l], t->ex.max_red[l]);
            ex.max_iter[l] = std::max(ex.max_iter[l], t->ex.max_iter[l]);
        }
        layouts[t->cfg.voxel_layout] = 1;
    }
    ex.ray_tw = b->ray_tw;
    // The captured tick reads its sessions from the device views, uploaded every
    // tick; it depends only on the slot count, the size extents and the voxel
    // layouts.  A session replaced by one of the same shape (serving churn)
    // keeps the graphs, and the tuner keeps its choice.
    if (nslots != b->nslots || memcmp(&ex, &b->ex, sizeof(ex)) != 0 ||
        memcmp(layouts, b->layouts, sizeof(layouts)) != 0) {
        batch_invalidate(b);
        b->tune_state = 0;  // a new shape: look it up or explore it at the next tick
        b->tick_cand[0] = b->tick_cand[1] = -1;
    }
    b->nslots = nslots;
    b->ex = ex;
    memcpy(b->layouts, layouts, sizeof(layouts));
}

GBF_API gbf_status gbf_batch_reserve(gbf_batch *b, const gbf_config *cfg, const gbf_intrinsics *K, int32_t slots) {
    if (!b || slots < 0 || slots > b->max_slots) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_reserve: bad slots");
    if (slots > 0) {
        gbf_status st = validate(cfg, K);
        if (st != GBF_OK) return st;
    }
    std::lock_guard<std::mutex> lock(b->mu);
    gbf_status fs = batch_flush(b, nullptr);
    if (fs != GBF_OK) return fs;
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) cudaEventSynchronize(b->ev[k]);
    Extent ex;
    memset(&ex, 0, sizeof(ex));
    memset(b->floor_layouts, 0, sizeof(b->floor_layouts));
    if (slots > 0) {  // the extents gbf_session_create gives a session of (cfg, K)
        ex.w = K->width;
        ex.h = K->height;
        ex.max_pool = cfg->num_blocks;
        ex.levels = cfg->num_levels;
        for (int l = 0; l < cfg->num_levels; ++l) {
            const int pw = K->width >> l, ph = K->height >> l, tile = reduce_tile(l);
            ex.max_red[l] = std::max(1, (pw * ph + tile - 1) / tile);
            ex.max_iter[l] = cfg->max_iterations[l];
        }
        b->floor_layouts[cfg->voxel_layout] = 1;
    }
    b->floor_ex = ex;
    b->floor_slots = slots;
    batch_reshape(b);
    return GBF_OK;
}

static void harvest(gbf_batch *b, int k) {
    float ms[kPhases];
    for (int i = 0; i < kPhases; ++i)
        if (cudaEventElapsedTime(&ms[i], b->pev[k][i], b->pev[k][i + 1]) != cudaSuccess) return;
    for (int i = 0; i < kPhases; ++i) b->phase_sum[i] += ms[i];
    b->phase_n += 1;
    b->pending[k] = 0;
}

// One tick.  With groups > 1 (and no phase timing) the slots are split into
// contiguous groups whose frames run as parallel branches (forked streams, or
// parallel graph branches when captured): sessions are independent, and the
// phases of one group (latency-bound reductions, issue-bound marching) fill
// the SMs another group's phase leaves idle.
static void batch_results(gbf_batch *b, int k, cudaStream_t st) {
    launch_slot_results(b->d_views, b->nslots, b->d_res[k], st);
    cudaMemcpyAsync(b->h_res[k], b->d_res[k], sizeof(gbf_slot_result) * b->nslots, cudaMemcpyDeviceToHost, st);
}

static int effective_groups(const gbf_batch *b) { return b->timing ? 1 : std::min(b->groups, b->nslots); }
static bool staggered(const gbf_batch *b) { return b->stagger && effective_groups(b) >= 2; }
static int group_lo(const gbf_batch *b, int g, int groups) { return b->nslots * g / groups; }

static void batch_enqueue(gbf_batch *b, int k, cudaStream_t st) {
    cudaMemcpyAsync(b->d_views, b->h_views[k], sizeof(SessionView) * b->nslots, cudaMemcpyHostToDevice, st);
    IngestArgs a{0, 0, nullptr, 0, nullptr, 0};
    const int groups = effective_groups(b);
    const bool stag = staggered(b);
    if (stag)
        cudaMemcpyAsync(b->d_views_b, b->h_views_b[k], sizeof(SessionView) * b->nslots, cudaMemcpyHostToDevice, st);
    if (groups <= 1) {
        enqueue_frame(b->d_views, b->nslots, b->ex, b->layouts, a, st, b->timing ? b->pev[k] : nullptr);
        batch_results(b, k, st);
        return;
    }
    cudaEventRecord(b->fork, st);
    for (int g = 1; g < groups; ++g) cudaStreamWaitEvent(b->side[g - 1], b->fork, 0);
    for (int g = 0; g < groups; ++g) {
        const int lo = group_lo(b, g, groups), hi = group_lo(b, g + 1, groups);
        cudaStream_t gs = g == 0 ? st : b->side[g - 1];
        if (stag && (g & 1)) {
            // half a frame out of phase: the previous frame's fusion and raycast,
            // then this frame's ingest and tracking, so that this group's tracking
            // runs beside the even groups' fusion and raycast and the other way round
            enqueue_second_half(b->d_views_b + lo, hi - lo, b->ex, b->layouts, gs);
            enqueue_first_half(b->d_views + lo, hi - lo, b->ex, a, gs);
        } else {
            enqueue_frame(b->d_views + lo, hi - lo, b->ex, b->layouts, a, gs);
        }
    }
    for (int g = 1; g < groups; ++g) {
        cudaEventRecord(b->join[g - 1], b->side[g - 1]);
        cudaStreamWaitEvent(st, b->join[g - 1], 0);
    }
    batch_results(b, k, st);
}

// Run the second halves the staggered groups owe (their last frames' fusion and
// raycast) and wait for them.  Called before anything that changes the slot
// assignment or the tick layout, and by gbf_batch_flush.
static gbf_status batch_flush(gbf_batch *b, cudaStream_t st) {
    bool any = false;
    for (int i = 0; i < b->nslots; ++i) any = any || b->owed[i];
    if (!any) return GBF_OK;
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) {
            cudaError_t e = cudaEventSynchronize(b->ev[k]);
            if (e != cudaSuccess) return cuda_error(e, "gbf_batch_flush: wait");
        }
    SessionView *hv = b->h_views_b[0];
    for (int i = 0; i < b->nslots; ++i) {
        if (b->owed[i] && b->sessions[i]) {
            hv[i] = b->sessions[i]->view;
            hv[i].active = 1;
        } else {
            memset(&hv[i], 0, sizeof(SessionView));
        }
    }
    cudaError_t e = cudaMemcpyAsync(b->d_views_b, hv, sizeof(SessionView) * b->nslots, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_batch_flush");
    enqueue_second_half(b->d_views_b, b->nslots, b->ex, b->layouts, st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_batch_flush");
    std::fill(b->owed.begin(), b->owed.end(), 0);
    return check_cuda("gbf_batch_flush");
}

GBF_API gbf_status gbf_batch_flush(gbf_batch *b, void *stream) {
    if (!b) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_flush: null");
    std::lock_guard<std::mutex> lock(b->mu);
    return batch_flush(b, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Online autotuner of the tick's launch shape.  Its knobs change how a tick is
// launched, never what it computes: the session groups (parallel branches),
// staggered groups, and the raycast tile.  While exploring, the batch serves
// as usual and times each tick with CUDA events on its stream; each candidate
// gets tune_ticks timed ticks (the first tick after a switch is not timed: it
// captures and uploads a new graph).  Coordinate search: groups x stagger at
// the 8-wide tile, then the tile at the best of those.  The fastest median is
// kept and recorded for the batch's shape in a process-wide table, which later
// batches of the same shape settle from without exploring.

namespace {

struct TuneKey {
    int device, nslots;
    Extent ex;  // ray_tw zeroed
    int layouts[kNumLayouts];
};

std::mutex g_tune_mu;
std::vector<std::pair<TuneKey, gbf_batch::Shape>> g_tune_table;

TuneKey tune_key(const gbf_batch *b) {
    TuneKey k;
    memset(&k, 0, sizeof(k));
    cudaGetDevice(&k.device);
    k.nslots = b->nslots;
    k.ex = b->ex;
    k.ex.ray_tw = 0;
    memcpy(k.layouts, b->layouts, sizeof(k.layouts));
    return k;
}

bool tune_lookup(const gbf_batch *b, gbf_batch::Shape *out) {
    const TuneKey k = tune_key(b);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (const auto &e : g_tune_table)
        if (memcmp(&e.first, &k, sizeof(k)) == 0) {
            *out = e.second;
            return true;
        }
    return false;
}

void tune_store(const gbf_batch *b, const gbf_batch::Shape &c) {
    const TuneKey k = tune_key(b);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (auto &e : g_tune_table)
        if (memcmp(&e.first, &k, sizeof(k)) == 0) {
            e.second = c;
            return;
        }
    const std::pair<TuneKey, gbf_batch::Shape> entry(k, c);
    g_tune_table.push_back(entry);
}

float median_ms(std::vector<float> v) {
    if (v.empty()) return FLT_MAX;
    std::sort(v.begin(), v.end());
    const size_t n = v.size();
    return (n & 1) ? v[n / 2] : 0.5f * (v[n / 2 - 1] + v[n / 2]);
}

int tune_best(const gbf_batch *b) {
    int best = 0;
    float best_ms = FLT_MAX;
    for (size_t i = 0; i < b->tune_cand.size(); ++i) {
        const float m = median_ms(b->tune_ms[i]);
        if (m < best_ms) {
            best_ms = m;
            best = (int)i;
        }
    }
    return best;
}

// The time of the tick last recorded on parity k, if it has ended (or, with
// wait, once it has).
void tune_collect(gbf_batch *b, int k, bool wait) {
    const int c = b->tick_cand[k];
    if (c < 0 || c >= (int)b->tune_ms.size()) return;
    if (!wait && cudaEventQuery(b->tev[k][1]) != cudaSuccess) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, b->tev[k][0], b->tev[k][1]) == cudaSuccess) b->tune_ms[c].push_back(ms);
    b->tick_cand[k] = -1;
}

// Switch the launch shape: owed halves run, ticks in flight end, graphs go.
gbf_status apply_shape(gbf_batch *b, const gbf_batch::Shape &c, cudaStream_t st) {
    if (c.groups == b->groups && c.stagger == b->stagger && c.ray_tw == b->ray_tw) return GBF_OK;
    gbf_status fs = batch_flush(b, st);
    if (fs != GBF_OK) return fs;
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) {
            cudaError_t e = cudaEventSynchronize(b->ev[k]);
            if (e != cudaSuccess) return cuda_error(e, "gbf_batch autotune: wait");
            tune_collect(b, k, true);
        }
    batch_invalidate(b);
    b->groups = c.groups;
    b->stagger = c.stagger;
    b->ray_tw = c.ray_tw;
    b->ex.ray_tw = c.ray_tw;
    return GBF_OK;
}

gbf_status tune_step(gbf_batch *b, cudaStream_t st) {
    if (!b->tune_on || b->timing || b->tune_state == 2) return GBF_OK;
    if (b->tune_state == 0) {
        gbf_batch::Shape c;
        if (tune_lookup(b, &c)) {
            b->tune_cached = 1;
            b->tune_state = 2;
            return apply_shape(b, c, st);
        }
        b->tune_cached = 0;
        b->tune_stage = 0;
        b->tune_cand.clear();
        for (int g = 1; g <= std::min(gbf_batch::kMaxGroups, b->nslots); ++g) {
            b->tune_cand.push_back({g, 0, 8});
            if (g >= 2) b->tune_cand.push_back({g, 1, 8});
        }
        b->tune_ms.assign(b->tune_cand.size(), std::vector<float>());
        b->tick_cand[0] = b->tick_cand[1] = -1;
        b->tune_cur = 0;
        b->tune_skip = 1;
        b->tune_state = 1;
        return apply_shape(b, b->tune_cand[0], st);
    }
    for (int k = 0; k < 2; ++k) tune_collect(b, k, false);
    if ((int)b->tune_ms[b->tune_cur].size() < b->tune_ticks) return GBF_OK;
    b->tune_cur += 1;
    if (b->tune_cur == (int)b->tune_cand.size()) {
        const gbf_batch::Shape best = b->tune_cand[tune_best(b)];
        if (b->tune_stage == 0) {
            for (int tw : {4, 16, 32}) {
                b->tune_cand.push_back({best.groups, best.stagger, tw});
                b->tune_ms.emplace_back();
            }
            b->tune_stage = 1;
        } else {
            tune_store(b, best);
            b->tune_state = 2;
            return apply_shape(b, best, st);
        }
    }
    b->tune_skip = 1;
    return apply_shape(b, b->tune_cand[b->tune_cur], st);
}

}  // namespace

GBF_API gbf_status gbf_batch_process(gbf_batch *b, const uint8_t *active, int32_t use_graph, void *stream) {
    if (!b || !active) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_process: null");
    std::lock_guard<std::mutex> lock(b->mu);
    if (b->nslots == 0) return GBF_OK;
    {
        gbf_status ts = tune_step(b, (cudaStream_t)stream);
        if (ts != GBF_OK) return ts;
    }
    const bool stag = staggered(b);
    if (!stag) {  // owed halves from a staggered tick run first
        gbf_status fs = batch_flush(b, (cudaStream_t)stream);
        if (fs != GBF_OK) return fs;
    }
    // work goes to `stream` (NULL = legacy default stream); graphs are captured
    // on the batch's own stream because the legacy stream cannot be captured
    cudaStream_t st = (cudaStream_t)stream;
    const int k = b->flip;
    b->flip ^= 1;
    if (b->ev_used[k]) {
        cudaError_t e = cudaEventSynchronize(b->ev[k]);
        if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: wait");
        if (b->timing && b->pending[k]) harvest(b, k);
        tune_collect(b, k, true);
    }
    SessionView *hv = b->h_views[k];
    for (int i = 0; i < b->nslots; ++i) {
        if (b->sessions[i]) {
            hv[i] = b->sessions[i]->view;
            hv[i].active = active[i] ? 1 : 0;
            if (b->staged[k][i]) {
                hv[i].in_depth = b->stg_depth[k][i];
                hv[i].in_rgb = b->stg_rgb[k][i];
                cudaError_t e = cudaStreamWaitEvent(st, b->staged_ev[k][i], 0);
                if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: wait for staging");
                b->staged[k][i] = 0;
            } else if (b->in_depth[i]) {
                hv[i].in_depth = b->in_depth[i];
                hv[i].in_rgb = b->in_rgb[i];
            }
        } else {
            memset(&hv[i], 0, sizeof(SessionView));
        }
    }
    if (stag) {
        SessionView *hb = b->h_views_b[k];
        for (int i = 0; i < b->nslots; ++i) {
            if (b->owed[i] && b->sessions[i]) {
                hb[i] = b->sessions[i]->view;
                hb[i].active = 1;
            } else {
                memset(&hb[i], 0, sizeof(SessionView));
            }
        }
    }
    // a tick timed for the tuner: events on the submitting stream around it
    const bool timed = b->tune_on && b->tune_state == 1 && !b->timing;
    b->tick_cand[k] = -1;
    if (timed) {
        if (b->tune_skip > 0) {
            b->tune_skip -= 1;
        } else {
            b->tick_cand[k] = b->tune_cur;
            cudaError_t e = cudaEventRecord(b->tev[k][0], st);
            if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: tuner event");
        }
    }
    if (use_graph) {
        if (!b->exec[k]) {
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(b->own, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: begin capture");
            batch_enqueue(b, k, b->own);
            e = cudaStreamEndCapture(b->own, &g);
            if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: end capture");
            e = cudaGraphInstantiate(&b->exec[k], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: instantiate");
            b->captures += 1;
        }
        cudaError_t e = cudaGraphLaunch(b->exec[k], st);
        if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: launch");
    } else {
        batch_enqueue(b, k, st);
    }
    if (b->tick_cand[k] >= 0) {
        cudaError_t e = cudaEventRecord(b->tev[k][1], st);
        if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: tuner event");
    }
    cudaError_t e = cudaEventRecord(b->ev[k], st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_batch_process: record");
    b->ev_used[k] = true;
    b->pending[k] = b->timing;
    b->last = k;
    b->submitted += 1;
    if (stag) {  // odd groups now owe this frame's second half
        const int groups = effective_groups(b);
        for (int g = 0; g < groups; ++g)
            for (int i = group_lo(b, g, groups); i < group_lo(b, g + 1, groups); ++i)
                b->owed[i] = (g & 1) && b->sessions[i] && active[i];
    }
    return check_cuda("gbf_batch_process");
}

GBF_API gbf_status gbf_batch_stage(gbf_batch *b, int32_t slot, const uint16_t *depth, int64_t depth_pitch,
                                   const uint8_t *rgb, int64_t rgb_pitch, void *stream) {
    if (!b || slot < 0 || slot >= b->max_slots || !depth || !rgb)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_stage: bad slot or pointers");
    std::lock_guard<std::mutex> lock(b->mu);
    gbf_session *s = b->sessions[slot];
    if (!s) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_stage: empty slot");
    const int W = s->K.width, H = s->K.height;
    if (depth_pitch < W * 2 || rgb_pitch < W * 3)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_stage: pitch smaller than a row");
    const int k = b->flip;  // parity of the next tick
    cudaError_t e = cudaSuccess;
    const size_t px = (size_t)W * H;
    if (b->stg_pixels[k][slot] != px) {  // first use of the slot, or a session of another size
        if (b->ev_used[k]) e = cudaEventSynchronize(b->ev[k]);
        if (b->stg_depth[k][slot]) cudaFree(b->stg_depth[k][slot]);
        if (b->stg_rgb[k][slot]) cudaFree(b->stg_rgb[k][slot]);
        b->stg_depth[k][slot] = nullptr;
        b->stg_rgb[k][slot] = nullptr;
        b->stg_pixels[k][slot] = 0;
        if (e == cudaSuccess) e = cudaMalloc(&b->stg_depth[k][slot], px * 2);
        if (e == cudaSuccess) e = cudaMalloc(&b->stg_rgb[k][slot], px * 3);
        if (e == cudaSuccess && !b->staged_ev[k][slot])
            e = cudaEventCreateWithFlags(&b->staged_ev[k][slot], cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_error(e, "gbf_batch_stage: buffers");
        b->stg_pixels[k][slot] = px;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // the tick two submissions back read these buffers
    if (b->ev_used[k]) e = cudaStreamWaitEvent(st, b->ev[k], 0);
    if (e == cudaSuccess) e = copy_rows(b->stg_depth[k][slot], depth, depth_pitch, (size_t)W * 2, H, st);
    if (e == cudaSuccess) e = copy_rows(b->stg_rgb[k][slot], rgb, rgb_pitch, (size_t)W * 3, H, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->staged_ev[k][slot], st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_batch_stage");
    b->staged[k][slot] = 1;
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_results(gbf_batch *b, int32_t back, gbf_slot_result *out, int32_t n) {
    if (!b || !out || n < 0 || back < 0 || back > 1)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_results: bad arguments");
    std::lock_guard<std::mutex> lock(b->mu);
    if (b->submitted <= back) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_results: no such tick");
    const int k = back == 0 ? b->last : (b->last ^ 1);
    cudaError_t e = cudaEventSynchronize(b->ev[k]);
    if (e != cudaSuccess) return cuda_error(e, "gbf_batch_results");
    memcpy(out, b->h_res[k], sizeof(gbf_slot_result) * std::min(n, b->nslots));
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_set_inputs(gbf_batch *b, int32_t slot, const uint16_t *depth_dev, const uint8_t *rgb_dev) {
    if (!b || slot < 0 || slot >= b->max_slots || (!depth_dev) != (!rgb_dev))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set_inputs: bad slot or pointers");
    std::lock_guard<std::mutex> lock(b->mu);
    b->in_depth[slot] = const_cast<uint16_t *>(depth_dev);
    b->in_rgb[slot] = const_cast<uint8_t *>(rgb_dev);
    return GBF_OK;
}

// A launch-shape knob set by hand ends the tuner's control of the batch.
static void tune_off(gbf_batch *b) {
    b->tune_on = 0;
    b->tune_state = 0;
    b->tick_cand[0] = b->tick_cand[1] = -1;
}

GBF_API gbf_status gbf_batch_set_groups(gbf_batch *b, int32_t groups) {
    if (!b || groups < 1 || groups > gbf_batch::kMaxGroups)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set_groups: 1..4 groups");
    std::lock_guard<std::mutex> lock(b->mu);
    gbf_status fs = batch_flush(b, nullptr);
    if (fs != GBF_OK) return fs;
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) cudaEventSynchronize(b->ev[k]);
    tune_off(b);
    if (groups != b->groups) batch_invalidate(b);
    b->groups = groups;
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_set_stagger(gbf_batch *b, int32_t enable) {
    if (!b) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set_stagger: null");
    std::lock_guard<std::mutex> lock(b->mu);
    gbf_status fs = batch_flush(b, nullptr);
    if (fs != GBF_OK) return fs;
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) cudaEventSynchronize(b->ev[k]);
    tune_off(b);
    if ((enable ? 1 : 0) != b->stagger) batch_invalidate(b);
    b->stagger = enable ? 1 : 0;
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_set_ray_tile(gbf_batch *b, int32_t tile_w) {
    if (!b || (tile_w != 4 && tile_w != 8 && tile_w != 16 && tile_w != 32))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set_ray_tile: tile width 4, 8, 16 or 32");
    std::lock_guard<std::mutex> lock(b->mu);
    gbf_status fs = batch_flush(b, nullptr);
    if (fs != GBF_OK) return fs;
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) cudaEventSynchronize(b->ev[k]);
    tune_off(b);
    if (tile_w != b->ray_tw) batch_invalidate(b);
    b->ray_tw = tile_w;
    b->ex.ray_tw = tile_w;
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_set_autotune(gbf_batch *b, int32_t enable, int32_t ticks_per_candidate) {
    if (!b) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set_autotune: null");
    std::lock_guard<std::mutex> lock(b->mu);
    if (enable && (ticks_per_candidate < 2 || ticks_per_candidate > 64))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set_autotune: 2..64 ticks per candidate");
    if (!enable) {
        tune_off(b);
        return GBF_OK;
    }
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 2; ++i)
            if (!b->tev[k][i]) {
                cudaError_t e = cudaEventCreate(&b->tev[k][i]);
                if (e != cudaSuccess) return cuda_error(e, "gbf_batch_set_autotune");
            }
    b->tune_on = 1;
    b->tune_ticks = ticks_per_candidate;
    b->tune_state = 0;
    b->tick_cand[0] = b->tick_cand[1] = -1;
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_tuning(gbf_batch *b, gbf_tuning *out) {
    if (!b || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_tuning: null");
    std::lock_guard<std::mutex> lock(b->mu);
    memset(out, 0, sizeof(*out));
    out->state = b->tune_on ? b->tune_state : 0;
    out->from_table = b->tune_on && b->tune_state == 2 ? b->tune_cached : 0;
    out->chosen.groups = b->groups;
    out->chosen.stagger = b->stagger;
    out->chosen.ray_tile_w = b->ray_tw;
    out->chosen.median_ms = 0.f;
    out->ticks_per_candidate = b->tune_ticks;
    if (b->tune_on && !b->tune_cached) {
        const int n = std::min((int)b->tune_cand.size(), GBF_TUNE_MAX_REPORT);
        out->n_tried = 0;
        for (int i = 0; i < n; ++i) {
            if (b->tune_ms[i].empty()) continue;
            gbf_launch_shape &t = out->tried[out->n_tried++];
            t.groups = b->tune_cand[i].groups;
            t.stagger = b->tune_cand[i].stagger;
            t.ray_tile_w = b->tune_cand[i].ray_tw;
            t.median_ms = median_ms(b->tune_ms[i]);
            if (t.groups == b->groups && t.stagger == b->stagger && t.ray_tile_w == b->ray_tw)
                out->chosen.median_ms = t.median_ms;
        }
    }
    return GBF_OK;
}

GBF_API gbf_status gbf_autotune_forget(void) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_table.clear();
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_set_timing(gbf_batch *b, int32_t enable) {
    if (!b) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_set_timing: null");
    std::lock_guard<std::mutex> lock(b->mu);
    gbf_status fs = batch_flush(b, nullptr);
    if (fs != GBF_OK) return fs;
    for (int k = 0; k < 2; ++k)
        if (b->ev_used[k]) cudaEventSynchronize(b->ev[k]);
    if (enable && !b->pev[0][0]) {
        for (int k = 0; k < 2; ++k)
            for (int i = 0; i <= kPhases; ++i) {
                cudaError_t e = cudaEventCreate(&b->pev[k][i]);
                if (e != cudaSuccess) return cuda_error(e, "gbf_batch_set_timing");
            }
    }
    b->timing = enable ? 1 : 0;
    b->pending[0] = b->pending[1] = 0;
    for (int i = 0; i < 8; ++i) b->phase_sum[i] = 0;
    b->phase_n = 0;
    batch_invalidate(b);
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_phase_ms(gbf_batch *b, float *ms, int32_t n) {
    if (!b || !ms || n < kPhases) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_phase_ms: need 7 floats");
    std::lock_guard<std::mutex> lock(b->mu);
    if (!b->timing) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_phase_ms: timing not enabled");
    for (int k = 0; k < 2; ++k)
        if (b->pending[k]) {
            cudaError_t e = cudaEventSynchronize(b->pev[k][kPhases]);
            if (e != cudaSuccess) return cuda_error(e, "gbf_batch_phase_ms");
            harvest(b, k);
        }
    for (int i = 0; i < kPhases; ++i) ms[i] = b->phase_n ? (float)(b->phase_sum[i] / b->phase_n) : 0.f;
    if (n > kPhases) ms[kPhases] = (float)b->phase_n;
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_captures(gbf_batch *b, int64_t *n) {
    if (!b || !n) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_captures: null");
    std::lock_guard<std::mutex> lock(b->mu);
    *n = b->captures;
    return GBF_OK;
}

GBF_API gbf_status gbf_batch_kernels(gbf_batch *b, int32_t *n) {
    if (!b || !n) return set_error(GBF_ERR_INVALID_ARG, "gbf_batch_kernels: null");
    std::lock_guard<std::mutex> lock(b->mu);
    int total = 0;
    const int groups = std::max(1, std::min(b->groups, b->nslots));
    for (int g = 0; g < groups; ++g)
        total += kernels_per_frame(b->ex, b->layouts, b->nslots * (g + 1) / groups - b->nslots * g / groups);
    *n = b->nslots ? total + 1 : 0;
    return GBF_OK;
}

}  // extern "C"
