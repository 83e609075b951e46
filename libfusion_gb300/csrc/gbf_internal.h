// gbf_internal.h -- host runtime internals (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "../../include/gbfusion.h"
#include "gbf_kernels.h"
#include "gbf_types.h"

namespace gbf {

struct M34Host {
    float m[12];
};

gbf_status set_error(gbf_status st, const char *msg);
gbf_status cuda_error(cudaError_t e, const char *where);
// cudaGetLastError after a launch sequence
gbf_status check_cuda(const char *where);

// Byte layout of one session's device arena.
struct ArenaLayout {
    size_t total;
    size_t table, bcoord, bstamp, bfresh, vis, mesh_off, vox_sw, vox_rgb, ctr, ts;
    size_t in_depth, in_rgb, depth_raw, rgb4, nmap_ext, fuse_px, zr_min, zr_max, partials;
    size_t depth[kMaxLevels], inten[2][kMaxLevels], gx[kMaxLevels], gy[kMaxLevels];
    size_t vmap[2][kMaxLevels], nmap[2][kMaxLevels], igd[2][kMaxLevels];
};

gbf_status validate(const gbf_config *cfg, const gbf_intrinsics *K);
ArenaLayout plan_arena(const gbf_config &cfg, const gbf_intrinsics &K);
int reduce_ctas(int pixels);
// reference pixels per reduction CTA at a pyramid level
int reduce_tile(int level);
// empty the session's map (table, pool, counters) but keep its pose and tracking state; synchronises
gbf_status reset_map(gbf_session *s);
// clear the table and insert every pool block [0, used) at its own id (gc.cu)
void rebuild_table(gbf_session *s, cudaStream_t st);

}  // namespace gbf

struct gbf_session {
    gbf_config cfg;
    gbf_intrinsics K;
    void *arena = nullptr;
    gbf::ArenaLayout lay;
    gbf::SessionView view;            // host copy (active = 1)
    gbf::SessionView *d_view = nullptr; // device copy for single-session launches
    gbf::Extent ex{};
    int layouts[gbf::kNumLayouts] = {};
    int device = 0;
};

struct gbf_batch {
    std::mutex mu;  // held by every gbf_batch_* call: a batch may be driven from several threads
    int max_slots = 0;
    std::vector<gbf_session *> sessions;
    std::vector<uint16_t *> in_depth;  // per-slot input override (device, dense)
    std::vector<uint8_t *> in_rgb;
    gbf::SessionView *h_views[2] = {nullptr, nullptr}; // pinned mirrors (ping-pong)
    gbf::SessionView *d_views = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool ev_used[2] = {false, false};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    cudaStream_t own = nullptr;
    int flip = 0;
    int nslots = 0;
    gbf::Extent ex{};
    int layouts[gbf::kNumLayouts] = {};
    int timing = 0;
    int last = -1;
    cudaEvent_t pev[2][8] = {};   // phase boundaries per mirror (captured into the graphs)
    int pending[2] = {0, 0};      // phase events recorded but not yet read
    double phase_sum[8] = {};
    long long phase_n = 0;
    // batch-owned input buffers per tick parity and slot (gbf_batch_stage)
    std::vector<uint16_t *> stg_depth[2];
    std::vector<uint8_t *> stg_rgb[2];
    std::vector<size_t> stg_pixels[2];
    std::vector<char> staged[2];                    // slot staged for the tick of this parity
    std::vector<cudaEvent_t> staged_ev[2];          // end of the slot's staging copy
    gbf_slot_result *d_res[2] = {nullptr, nullptr}; // per-slot results of the tick (device)
    gbf_slot_result *h_res[2] = {nullptr, nullptr}; // pinned copies
    long long submitted = 0;                        // ticks submitted
    // staggered groups: odd groups run the second half of their previous frame
    // and then the first half of this one in each tick
    int stagger = 0;
    gbf::SessionView *h_views_b[2] = {nullptr, nullptr}; // second-half views (active = half owed)
    gbf::SessionView *d_views_b = nullptr;
    std::vector<char> owed;                         // slot owes the second half of its last frame
    static constexpr int kMaxGroups = 4;
    int groups = 2;                                // concurrent session groups per tick
    cudaStream_t side[kMaxGroups - 1] = {};        // branch streams of groups 1..
    cudaEvent_t fork = nullptr, join[kMaxGroups - 1] = {};
    int ray_tw = 8;                                // raycast tile width (64-pixel tiles)
    // online autotuner of the launch shape (groups, stagger, raycast tile)
    struct Shape {
        int groups, stagger, ray_tw;
    };
    int tune_on = 0;                    // gbf_batch_set_autotune
    int tune_state = 0;                 // 0 idle, 1 exploring, 2 settled
    int tune_ticks = 6;                 // timed ticks per candidate
    int tune_stage = 0;                 // 0: groups x stagger at an 8-wide tile, 1: the tile
    int tune_cur = -1;                  // candidate being timed
    int tune_skip = 0;                  // ticks left to skip after a switch
    int tune_cached = 0;                // settled from the process-wide table
    std::vector<Shape> tune_cand;
    std::vector<std::vector<float>> tune_ms;  // tick times (ms) per candidate
    cudaEvent_t tev[2][2] = {};         // per tick parity: start, end of the tick
    int tick_cand[2] = {-1, -1};        // candidate the tick in flight was timed for
    // reserved shape (gbf_batch_reserve): the tick's extents and slot count never
    // fall below these, so sessions up to it come and go without a new graph
    gbf::Extent floor_ex{};
    int floor_slots = 0;
    int floor_layouts[gbf::kNumLayouts] = {};
    long long captures = 0;             // tick graphs captured (gbf_batch_captures)
};
