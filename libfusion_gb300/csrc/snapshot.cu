// snapshot.cu -- session snapshot and restore: evict a serving session to host
// memory and resume it later, bit for bit.
//
// The reference keeps one map per process and can only dump the map storage
// (MapStruct::writeToDisk, src/data_struct/map_struct.cu:534-613; no pose, no
// tracking state).  A snapshot here holds everything the next frame reads:
//
//   header        magic, format version, the session's configuration and
//                 intrinsics (a restore needs the same), block count, size
//   track state   poses, the tracker's state, the motion prior, frame index
//   counters      pool end, frame stamp, status bits
//   blocks        coordinates, stamps, fresh bits, and the voxels and colours
//                 of blocks [0, used) in the session's own storage layout
//                 (no conversion, block ids kept)
//   reference     the reference frame's pyramid: the raycast prediction's
//                 vertex and normal maps and the intensity of every level
//
// Everything else a frame reads is rewritten by that frame's ingest.  The hash
// table is not stored: a restore re-inserts the blocks at their ids.  Sections
// start on 256-byte boundaries so that a snapshot in device memory copies
// with aligned transfers.
#include <algorithm>
#include <cstring>

#include "gbf_internal.h"

namespace gbf {
namespace {

constexpr char kMagic[8] = {'G', 'B', 'F', 'S', 'N', 'A', 'P', '\0'};
constexpr uint32_t kVersion = 1;

struct SnapHeader {
    char magic[8];
    uint32_t version;
    uint32_t track_state_bytes;
    gbf_config cfg;
    gbf_intrinsics K;
    int64_t n_blocks;
    int64_t total_bytes;
};

struct SnapLayout {
    size_t ts, ctr, bcoord, bstamp, bfresh, vox_sw, vox_rgb;
    size_t vmap[kMaxLevels], nmap[kMaxLevels], inten[kMaxLevels];
    size_t pixels[kMaxLevels];
    size_t total;
};

size_t voxel_sw_bytes(const gbf_config &c) { return c.voxel_layout == GBF_VOXEL_REF ? 8 : 4; }

SnapLayout snap_layout(const gbf_config &c, const gbf_intrinsics &K, int64_t n) {
    SnapLayout L;
    memset(&L, 0, sizeof(L));
    size_t off = 0;
    auto take = [&](size_t bytes) {
        off = (off + 255) & ~size_t(255);
        const size_t o = off;
        off += bytes;
        return o;
    };
    take(sizeof(SnapHeader));
    L.ts = take(sizeof(TrackState));
    L.ctr = take(C_COUNT * sizeof(int));
    L.bcoord = take((size_t)n * sizeof(int4));
    L.bstamp = take((size_t)n * sizeof(int));
    L.bfresh = take((size_t)n);
    L.vox_sw = take((size_t)n * kBlockVoxels * voxel_sw_bytes(c));
    L.vox_rgb = take((size_t)n * kBlockVoxels * 4);
    size_t w = K.width, h = K.height;
    for (int l = 0; l < c.num_levels; ++l) {
        L.pixels[l] = w * h;
        L.vmap[l] = take(w * h * 16);
        L.nmap[l] = take(w * h * 16);
        L.inten[l] = take(w * h * 4);
        w /= 2;
        h /= 2;
    }
    L.total = (off + 255) & ~size_t(255);
    return L;
}

// blocks [0, used) of the pool, read from the device (synchronises)
gbf_status used_blocks_host(gbf_session *s, cudaStream_t st, int64_t *n, TrackState *ts, const char *what) {
    int used = 0;
    cudaError_t e = cudaMemcpyAsync(&used, s->view.ctr + C_NUSED, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && ts) e = cudaMemcpyAsync(ts, s->view.ts, sizeof(TrackState), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, what);
    *n = std::min(used, s->cfg.num_blocks);
    return GBF_OK;
}

}  // namespace
}  // namespace gbf

using namespace gbf;

extern "C" {

GBF_API gbf_status gbf_session_snapshot_bytes(gbf_session *s, int64_t *bytes) {
    if (!s || !bytes) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_snapshot_bytes: null");
    cudaError_t e = cudaDeviceSynchronize();  // the pool end after every queued frame
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_snapshot_bytes");
    int64_t n = 0;
    gbf_status st = used_blocks_host(s, nullptr, &n, nullptr, "gbf_session_snapshot_bytes");
    if (st != GBF_OK) return st;
    *bytes = (int64_t)snap_layout(s->cfg, s->K, n).total;
    return GBF_OK;
}

GBF_API gbf_status gbf_session_snapshot(gbf_session *s, void *dst, int64_t capacity, int64_t *written, void *stream) {
    if (!s || !dst) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_snapshot: null");
    cudaStream_t st = (cudaStream_t)stream;
    int64_t n = 0;
    TrackState ts;
    gbf_status r = used_blocks_host(s, st, &n, &ts, "gbf_session_snapshot");
    if (r != GBF_OK) return r;
    const SnapLayout L = snap_layout(s->cfg, s->K, n);
    if (capacity < (int64_t)L.total) return set_error(GBF_ERR_CAPACITY, "gbf_session_snapshot: buffer too small");
    SnapHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kMagic, sizeof(kMagic));
    h.version = kVersion;
    h.track_state_bytes = sizeof(TrackState);
    h.cfg = s->cfg;
    h.K = s->K;
    h.n_blocks = n;
    h.total_bytes = (int64_t)L.total;
    char *d = static_cast<char *>(dst);
    const SessionView &v = s->view;
    const int ref = ts.idx;  // the reference image set
    struct Part {
        size_t off;
        const void *src;
        size_t bytes;
    };
    std::vector<Part> parts = {
        {0, &h, sizeof(h)},
        {L.ts, v.ts, sizeof(TrackState)},
        {L.ctr, v.ctr, C_COUNT * sizeof(int)},
        {L.bcoord, v.bcoord, (size_t)n * sizeof(int4)},
        {L.bstamp, v.bstamp, (size_t)n * sizeof(int)},
        {L.bfresh, v.bfresh, (size_t)n},
        {L.vox_sw, v.vox_sw, (size_t)n * kBlockVoxels * voxel_sw_bytes(s->cfg)},
        {L.vox_rgb, v.vox_rgb, (size_t)n * kBlockVoxels * 4},
    };
    for (int l = 0; l < s->cfg.num_levels; ++l) {
        parts.push_back({L.vmap[l], v.vmap[ref][l], L.pixels[l] * 16});
        parts.push_back({L.nmap[l], v.nmap[ref][l], L.pixels[l] * 16});
        parts.push_back({L.inten[l], v.inten[ref][l], L.pixels[l] * 4});
    }
    for (const Part &p : parts) {
        if (p.bytes == 0) continue;
        cudaError_t e = cudaMemcpyAsync(d + p.off, p.src, p.bytes, cudaMemcpyDefault, st);
        if (e != cudaSuccess) return cuda_error(e, "gbf_session_snapshot");
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_snapshot");
    if (written) *written = (int64_t)L.total;
    return check_cuda("gbf_session_snapshot");
}

GBF_API gbf_status gbf_session_restore(gbf_session *s, const void *src, int64_t bytes, void *stream) {
    if (!s || !src) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_restore: null");
    if (bytes < (int64_t)sizeof(SnapHeader)) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_restore: too short");
    cudaStream_t st = (cudaStream_t)stream;
    SnapHeader h;
    cudaError_t e = cudaMemcpy(&h, src, sizeof(h), cudaMemcpyDefault);
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_restore");
    if (memcmp(h.magic, kMagic, sizeof(kMagic)) != 0 || h.version != kVersion ||
        h.track_state_bytes != sizeof(TrackState))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_session_restore: not a snapshot of this library version");
    if (memcmp(&h.cfg, &s->cfg, sizeof(gbf_config)) != 0 || memcmp(&h.K, &s->K, sizeof(gbf_intrinsics)) != 0)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_session_restore: the session's configuration or intrinsics differ");
    if (h.n_blocks < 0 || h.n_blocks > s->cfg.num_blocks)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_session_restore: block count out of range");
    const int64_t n = h.n_blocks;
    const SnapLayout L = snap_layout(s->cfg, s->K, n);
    if (h.total_bytes != (int64_t)L.total || bytes < (int64_t)L.total)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_session_restore: size does not match the snapshot");
    TrackState ts;
    e = cudaMemcpy(&ts, static_cast<const char *>(src) + L.ts, sizeof(ts), cudaMemcpyDefault);
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_restore");
    if (ts.idx != 0 && ts.idx != 1) return set_error(GBF_ERR_INVALID_ARG, "gbf_session_restore: corrupt track state");
    int ctr[C_COUNT];
    e = cudaMemcpy(ctr, static_cast<const char *>(src) + L.ctr, sizeof(ctr), cudaMemcpyDefault);
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_restore");
    ctr[C_NUSED] = (int)n;
    ctr[C_NVIS] = 0;   // the visible list and render count of the last frame are not kept
    ctr[C_RENDER] = 0;
    ctr[C_TICKET] = 0;
    const char *sp = static_cast<const char *>(src);
    const SessionView &v = s->view;
    const int ref = ts.idx;
    struct Part {
        void *dst;
        size_t off, bytes;
    };
    std::vector<Part> parts = {
        {v.bcoord, L.bcoord, (size_t)n * sizeof(int4)},
        {v.bstamp, L.bstamp, (size_t)n * sizeof(int)},
        {v.bfresh, L.bfresh, (size_t)n},
        {v.vox_sw, L.vox_sw, (size_t)n * kBlockVoxels * voxel_sw_bytes(s->cfg)},
        {v.vox_rgb, L.vox_rgb, (size_t)n * kBlockVoxels * 4},
    };
    for (int l = 0; l < s->cfg.num_levels; ++l) {
        parts.push_back({v.vmap[ref][l], L.vmap[l], L.pixels[l] * 16});
        parts.push_back({v.nmap[ref][l], L.nmap[l], L.pixels[l] * 16});
        parts.push_back({v.inten[ref][l], L.inten[l], L.pixels[l] * 4});
    }
    for (const Part &p : parts) {
        if (p.bytes == 0) continue;
        e = cudaMemcpyAsync(p.dst, sp + p.off, p.bytes, cudaMemcpyDefault, st);
        if (e != cudaSuccess) return cuda_error(e, "gbf_session_restore");
    }
    e = cudaMemcpyAsync(v.ts, &ts, sizeof(ts), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v.ctr, ctr, sizeof(ctr), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_restore");
    rebuild_table(s, st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "gbf_session_restore");
    return check_cuda("gbf_session_restore");
}

}  // extern "C"
