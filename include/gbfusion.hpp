// gbfusion.hpp -- header-only C++ shim with the reference's class names and
// method set on top of the C ABI (gbfusion.h).  OpenCV, Sophus and Eigen are
// not required: images are DeviceImageView (device pointer + pitch + size)
// and poses are row-major 4x4 double matrices (Pose), the matrix form of the
// reference's Sophus::SE3d.
//
// Reference interfaces mirrored (paths relative to the reference project):
//   fusion::IntrinsicMatrix  include/data_struct/intrinsic_matrix.h:12-49
//   fusion::DenseMapping     include/voxel_hashing/voxel_hashing.h:12-51
//   fusion::DenseTracking    include/tracking/icp_tracker.h:28-88
//   fusion::DenseOdometry    include/tracking/rgbd_odometry.h:13-41
//   fusion::System           include/system.h:17-95
// fusion::FusionBatch (no counterpart in the reference) serves many sessions
// per launch: gbf_batch_* of gbfusion.h.
// Errors raise fusion::Error (the reference prints and exits the process,
// include/utils/safe_call.h:13-23).
#ifndef GBFUSION_HPP
#define GBFUSION_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbfusion.h"

namespace fusion {

struct Error : std::runtime_error {
    gbf_status status;
    Error(gbf_status s, const std::string &where)
        : std::runtime_error(where + ": " + gbf_last_error()), status(s) {}
};

inline void check(gbf_status s, const char *where) {
    if (s != GBF_OK) throw Error(s, where);
}

using Pose = std::array<double, 16>;  // row-major T_wc

inline Pose identity() { return Pose{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}; }

struct DeviceImageView {
    void *data = nullptr;
    int64_t pitch = 0;  // bytes per row
    int rows = 0, cols = 0;
};

struct IntrinsicMatrix {
    int width = 0, height = 0;
    float fx = 0, fy = 0, cx = 0, cy = 0, invfx = 0, invfy = 0;
    IntrinsicMatrix() = default;
    IntrinsicMatrix(int cols, int rows, float fx_, float fy_, float cx_, float cy_)
        : width(cols), height(rows), fx(fx_), fy(fy_), cx(cx_), cy(cy_), invfx(1.0f / fx_), invfy(1.0f / fy_) {}
    IntrinsicMatrix pyr_down() const {
        const float s = 0.5f;
        return IntrinsicMatrix((int)(s * width), (int)(s * height), s * fx, s * fy, s * cx, s * cy);
    }
    gbf_intrinsics c() const { return gbf_intrinsics{width, height, fx, fy, cx, cy}; }
};

inline gbf_config default_config() {
    gbf_config c;
    check(gbf_config_default(&c), "gbf_config_default");
    return c;
}

struct TrackingResult {
    bool sucess = false;  // (sic) the reference's field name
    float icp_error = 0;
    Pose update = identity();
};

// One session owns the map and the tracker state on the GPU.
class Session {
  public:
    Session(const IntrinsicMatrix &K, const gbf_config &cfg = default_config()) : K_(K), cfg_(cfg) {
        gbf_intrinsics k = K.c();
        gbf_session *s = nullptr;
        check(gbf_session_create(&cfg_, &k, &s), "gbf_session_create");
        s_.reset(s, [](gbf_session *p) { gbf_session_destroy(p); });
    }
    gbf_session *handle() const { return s_.get(); }
    std::shared_ptr<gbf_session> shared_handle() const { return s_; }
    const IntrinsicMatrix &intrinsics() const { return K_; }
    // the next frame from host or device memory, into the session's own input
    // buffers (for gbf_batch_process or gbf_process_frame_staged)
    void stage(const void *depth_mm, int64_t depth_pitch, const void *rgb, int64_t rgb_pitch, void *stream = nullptr) {
        check(gbf_session_stage(handle(), (const uint16_t *)depth_mm, depth_pitch, (const uint8_t *)rgb, rgb_pitch,
                                stream), "Session::stage");
    }
    const gbf_config &config() const { return cfg_; }

  protected:
    IntrinsicMatrix K_;
    gbf_config cfg_;
    std::shared_ptr<gbf_session> s_;
};

class DenseMapping : public Session {
  public:
    using Session::Session;
    // update(depth, image, pose): 1/d^2 colour update (voxel_hashing.cpp:67-85)
    void update(const DeviceImageView &depth, const DeviceImageView &image, const Pose &pose, void *stream = nullptr) {
        check(gbf_fuse(handle(), (const float *)depth.data, depth.pitch, (const uint8_t *)image.data, image.pitch,
                       nullptr, 0, pose.data(), stream), "DenseMapping::update");
    }
    // update(frame): normal-weighted update with the frame's level-0 normals (voxel_hashing.cpp:44-65)
    void update(const DeviceImageView &depth, const DeviceImageView &image, const DeviceImageView &normal,
                const Pose &pose, void *stream = nullptr) {
        check(gbf_fuse(handle(), (const float *)depth.data, depth.pitch, (const uint8_t *)image.data, image.pitch,
                       (const float *)normal.data, normal.pitch, pose.data(), stream), "DenseMapping::update");
    }
    void raycast(DeviceImageView &vmap, const Pose &pose, void *stream = nullptr) {
        check(gbf_raycast(handle(), pose.data(), (float *)vmap.data, vmap.pitch, stream), "DenseMapping::raycast");
    }
    // raycast(vmap, image, pose) (voxel_hashing.h:20): the vertex map plus the
    // hits' voxel colours (RGB888) in image; nmap, when given, the model normals
    void raycast(DeviceImageView &vmap, DeviceImageView &image, const Pose &pose, DeviceImageView *nmap = nullptr,
                 void *stream = nullptr) {
        check(gbf_raycast_maps(handle(), pose.data(), (float *)vmap.data, vmap.pitch,
                               nmap ? (float *)nmap->data : nullptr, nmap ? nmap->pitch : 0,
                               (uint8_t *)image.data, image.pitch, stream),
              "DenseMapping::raycast");
    }
    void reset_mapping(void *stream = nullptr) { check(gbf_session_reset(handle(), stream), "reset_mapping"); }
    // deleteBlock (map_struct.cu:327-363) for the listed block coordinates (x, y, z per
    // block); returns the blocks removed
    int64_t delete_blocks(const std::vector<int32_t> &coords) {
        int64_t n = 0;
        check(gbf_map_delete_blocks(handle(), coords.empty() ? nullptr : coords.data(), (int64_t)(coords.size() / 3),
                                    &n), "DenseMapping::delete_blocks");
        return n;
    }
    // the blocks farther than radius from center (nullptr: no distance test) and,
    // with drop_unobserved, those without an observed voxel; returns the blocks removed
    int64_t prune(const double *center, double radius, bool drop_unobserved = false) {
        int64_t n = 0;
        check(gbf_map_prune(handle(), center, radius, drop_unobserved ? 1 : 0, &n), "DenseMapping::prune");
        return n;
    }
    // prune() on `stream`, no host synchronisation (between the ticks of a batch)
    void prune_async(const double *center, double radius, bool drop_unobserved = false, void *stream = nullptr) {
        check(gbf_map_prune_async(handle(), center, radius, drop_unobserved ? 1 : 0, stream),
              "DenseMapping::prune_async");
    }
    // mesh buffers are caller-allocated device memory of max_tris triangles (system.h:36-41)
    size_t fetch_mesh_vertex_only(void *vertex, size_t max_tris) {
        uint64_t n = 0;
        check(gbf_extract_mesh(handle(), GBF_MESH_VERTEX, (float *)vertex, nullptr, max_tris, &n, nullptr),
              "fetch_mesh_vertex_only");
        return (size_t)n;
    }
    size_t fetch_mesh_with_normal(void *vertex, void *normal, size_t max_tris) {
        uint64_t n = 0;
        check(gbf_extract_mesh(handle(), GBF_MESH_NORMAL, (float *)vertex, normal, max_tris, &n, nullptr),
              "fetch_mesh_with_normal");
        return (size_t)n;
    }
    size_t fetch_mesh_with_colour(void *vertex, void *colour, size_t max_tris) {
        uint64_t n = 0;
        check(gbf_extract_mesh(handle(), GBF_MESH_COLOUR, (float *)vertex, colour, max_tris, &n, nullptr),
              "fetch_mesh_with_colour");
        return (size_t)n;
    }
    void raycast_check_visibility(DeviceImageView &vmap, const Pose &pose, void *stream = nullptr) {
        check(gbf_raycast_check_visibility(handle(), pose.data(), (float *)vmap.data, vmap.pitch, stream),
              "raycast_check_visibility");
    }
    // the reference's raw dump: file_name + file_name.txt (reference default sizes)
    void writeMapToDisk(const std::string &file_name) {
        check(gbf_map_write_dump(handle(), file_name.c_str(), nullptr), "writeMapToDisk");
    }
    void readMapFromDisk(const std::string &file_name) {
        check(gbf_map_read_dump(handle(), file_name.c_str()), "readMapFromDisk");
    }
};

class DenseTracking : public DenseMapping {
  public:
    using DenseMapping::DenseMapping;
    void set_source(const DeviceImageView &depth, const DeviceImageView &image, void *stream = nullptr) {
        check(gbf_build_pyramid(handle(), 0, (const float *)depth.data, depth.pitch, (const uint8_t *)image.data,
                                image.pitch, stream), "set_source");
    }
    void set_reference(const DeviceImageView &depth, const DeviceImageView &image, void *stream = nullptr) {
        check(gbf_build_pyramid(handle(), 1, (const float *)depth.data, depth.pitch, (const uint8_t *)image.data,
                                image.pitch, stream), "set_reference");
    }
    TrackingResult compute_transform(const Pose &init = identity(), void *stream = nullptr) {
        gbf_track_result r;
        check(gbf_track(handle(), init.data(), &r, stream), "compute_transform");
        TrackingResult t;
        t.sucess = r.success != 0;
        t.icp_error = r.icp_error;
        for (int i = 0; i < 16; ++i) t.update[i] = r.update[i];
        return t;
    }
};

// System::process_images: u16 depth (mm) + rgb8 in, pose out
class System : public DenseTracking {
  public:
    using DenseTracking::DenseTracking;
    void process_images(const DeviceImageView &depth_mm, const DeviceImageView &image, void *stream = nullptr) {
        check(gbf_process_frame(handle(), (const uint16_t *)depth_mm.data, depth_mm.pitch,
                                (const uint8_t *)image.data, image.pitch, stream), "process_images");
    }
    Pose get_camera_pose(void *stream = nullptr) const {
        Pose p;
        check(gbf_get_pose(handle(), p.data(), stream), "get_camera_pose");
        return p;
    }
    void set_pose(const Pose &p, void *stream = nullptr) { check(gbf_set_pose(handle(), p.data(), stream), "set_pose"); }
};

// Serving: the sessions in its slots advance one frame per tick, all in the
// same launches (a captured graph per tick shape).  The batch keeps every
// session it holds alive; it is destroyed (flushing what staggered groups owe)
// before it lets them go.
class FusionBatch {
  public:
    explicit FusionBatch(int max_sessions) : held_(max_sessions) {
        gbf_batch *b = nullptr;
        check(gbf_batch_create(max_sessions, &b), "gbf_batch_create");
        b_.reset(b, [](gbf_batch *p) { gbf_batch_destroy(p); });
    }
    gbf_batch *handle() const { return b_.get(); }
    // put a session into a slot (nullptr empties it)
    void set(int slot, const Session *s) {
        check(gbf_batch_set(handle(), slot, s ? s->handle() : nullptr), "FusionBatch::set");
        held_.at(slot) = s ? s->shared_handle() : nullptr;
    }
    // size the tick for `slots` sessions no larger than (cfg, K): sessions of up
    // to that size then come and go without a new captured graph
    void reserve(const gbf_config &cfg, const gbf_intrinsics &K, int slots) {
        check(gbf_batch_reserve(handle(), &cfg, &K, slots), "FusionBatch::reserve");
    }
    // tick graphs captured so far
    int64_t captures() {
        int64_t n = 0;
        check(gbf_batch_captures(handle(), &n), "FusionBatch::captures");
        return n;
    }
    // frames read from device memory at each tick (nullptr, nullptr: the session's staging)
    void set_inputs(int slot, const uint16_t *depth_dev, const uint8_t *rgb_dev) {
        check(gbf_batch_set_inputs(handle(), slot, depth_dev, rgb_dev), "FusionBatch::set_inputs");
    }
    // copy the next tick's frame (host or device memory) on `stream`, overlapping the running tick
    void stage(int slot, const void *depth_mm, int64_t depth_pitch, const void *rgb, int64_t rgb_pitch,
               void *stream = nullptr) {
        check(gbf_batch_stage(handle(), slot, (const uint16_t *)depth_mm, depth_pitch, (const uint8_t *)rgb,
                              rgb_pitch, stream), "FusionBatch::stage");
    }
    void process(const std::vector<uint8_t> &active, bool use_graph = true, void *stream = nullptr) {
        check(gbf_batch_process(handle(), active.data(), use_graph ? 1 : 0, stream), "FusionBatch::process");
    }
    // per-slot pose, tracking flag and status of the last tick (back = 0) or the one before
    std::vector<gbf_slot_result> results(int back = 0) {
        std::vector<gbf_slot_result> r(held_.size());
        check(gbf_batch_results(handle(), back, r.data(), (int32_t)r.size()), "FusionBatch::results");
        return r;
    }
    void set_groups(int groups) { check(gbf_batch_set_groups(handle(), groups), "FusionBatch::set_groups"); }
    void set_stagger(bool on) { check(gbf_batch_set_stagger(handle(), on ? 1 : 0), "FusionBatch::set_stagger"); }
    void set_ray_tile(int tile_w) { check(gbf_batch_set_ray_tile(handle(), tile_w), "FusionBatch::set_ray_tile"); }
    void autotune(bool on = true, int ticks_per_candidate = 6) {
        check(gbf_batch_set_autotune(handle(), on ? 1 : 0, ticks_per_candidate), "FusionBatch::autotune");
    }
    gbf_tuning tuning() const {
        gbf_tuning t;
        check(gbf_batch_tuning(handle(), &t), "FusionBatch::tuning");
        return t;
    }
    void flush(void *stream = nullptr) { check(gbf_batch_flush(handle(), stream), "FusionBatch::flush"); }

  private:
    std::vector<std::shared_ptr<gbf_session>> held_;  // declared first: released after the batch
    std::shared_ptr<gbf_batch> b_;
};

// DenseOdometry::trackFrame keeps the reference pyramid between frames; in this
// library that state lives in the session, so the odometry is the System's
// tracking half.
using DenseOdometry = System;

}  // namespace fusion

#endif
