// gc.cu -- block garbage collection on the device: deleteBlock
// (src/data_struct/map_struct.cu:327-363) for block lists and for blocks
// selected by distance or by carrying no observation.
//
// The reference's deleteBlock zeroes the block, returns its pool index to the
// heap and unlinks its hash entry under the bucket lock; it is defined but
// never called (its one caller is commented out, depth_fusion.cu:70), so the
// reference's pool only grows.  Here the pool is a dense range [0, used) and
// the table is open addressing, so a collection is a stream-ordered pass with
// no host round trip:
//
//   mark    keep flag per block (one warp per block)
//   scan    exclusive prefix of the flags (one CTA): K blocks kept
//   holes   the deleted positions below K, listed in order
//   move    each kept block at or above K moves into the next hole (voxels,
//           colours, coordinates, stamp): sources lie at or above K and
//           destinations below it, so no block is read after it is written
//   table   cleared and refilled with the K kept blocks; claimed slots whose
//           block the full pool had refused (ptr -1) go with it
//
// The keep flags and the scan live in the mesh offset array, the hole list in
// the visible list (both are rebuilt by the next mesh / fuse); the last fuse's
// visible list and render count are emptied, as its block ids no longer hold.
#include <algorithm>

#include "gbf_device.cuh"
#include "gbf_internal.h"

namespace gbf {
namespace {

constexpr int kGcThreads = 256;

struct GcArgs {
    int use_radius, drop_unobserved;
    double cx, cy, cz, r2, block_metres;
};

__device__ __forceinline__ int used_blocks(const SessionView &sv) { return min(sv.ctr[C_NUSED], sv.pool); }

// keep[id] = 1 unless the block's centre lies farther than the radius from the
// centre, or (drop_unobserved) no voxel of it carries a weight.  One warp per block.
template <int LAYOUT>
__global__ void gc_mark_kernel(const SessionView *__restrict__ svs, GcArgs a, int *keep) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int id = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); id < n; id += warps) {
        bool k = true;
        if (a.use_radius) {
            const int4 c = sv.bcoord[id];
            // block centre in double, the same operations in the same order for every block
            const double x = ((double)c.x + 0.5) * a.block_metres - a.cx;
            const double y = ((double)c.y + 0.5) * a.block_metres - a.cy;
            const double z = ((double)c.z + 0.5) * a.block_metres - a.cz;
            double d2 = 0.0;
            d2 += x * x;
            d2 += y * y;
            d2 += z * z;
            if (d2 > a.r2) k = false;
        }
        if (k && a.drop_unobserved) {
            bool seen = false;
            if (!sv.bfresh[id])  // a block not yet integrated holds zeros
                for (int i = lane; i < kBlockVoxels; i += 32)
                    seen = seen || load_vox<LAYOUT>(sv, (size_t)id * kBlockVoxels + i).w != 0.f;
            k = __any_sync(0xffffffffu, seen);
        }
        if (lane == 0) keep[id] = k ? 1 : 0;
    }
}

__global__ void gc_keep_all_kernel(const SessionView *__restrict__ svs, int *keep) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) keep[id] = 1;
}

// clear the flag of every listed block that is allocated (others are ignored)
__global__ void gc_unmark_list_kernel(const SessionView *__restrict__ svs, const int *coords, int m, int *keep) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const int id = find_block(sv, coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]);
        if (id >= 0 && id < n) keep[id] = 0;
    }
}

// Exclusive scan of keep[0..n) in place, keep[n] = K (blocks kept), and the
// number deleted into C_GC_DELETED.  One CTA of 1024 threads, 1024 flags per step.
__global__ void gc_scan_kernel(const SessionView *__restrict__ svs, int *keep) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    __shared__ int wsum[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < n ? keep[i] : 0;
        int x = v;  // inclusive warp scan
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int w = lane < nw ? wsum[lane] : 0;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        if (i < n) keep[i] = carry + (wid ? wsum[wid - 1] : 0) + (x - v);
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        keep[n] = carry;
        sv.ctr[C_GC_DELETED] = n - carry;
    }
}

// hole[r] = the r-th deleted position below K
__global__ void gc_holes_kernel(const SessionView *__restrict__ svs, const int *pre, int *hole) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    const int K = pre[n];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x)
        if (pre[i + 1] == pre[i]) hole[i - pre[i]] = i;
}

// Each kept block at or above K moves into the hole of its rank among them.
template <int LAYOUT>
__global__ void gc_move_kernel(const SessionView *__restrict__ svs, const int *pre, const int *hole) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    const int K = pre[n], kept_low = pre[K];
    constexpr int kWords = kBlockVoxels * (LAYOUT == GBF_VOXEL_REF ? 8 : 4) / 16;  // 16-byte words per block
    constexpr int kRgbWords = kBlockVoxels * 4 / 16;
    for (int i = K + blockIdx.x; i < n; i += gridDim.x) {
        if (pre[i + 1] == pre[i]) continue;  // deleted
        const int dst = hole[pre[i] - kept_low];
        const uint4 *s = reinterpret_cast<const uint4 *>(sv.vox_sw) + (size_t)i * kWords;
        uint4 *d = reinterpret_cast<uint4 *>(sv.vox_sw) + (size_t)dst * kWords;
        for (int w = threadIdx.x; w < kWords; w += blockDim.x) d[w] = s[w];
        const uint4 *sr = reinterpret_cast<const uint4 *>(sv.vox_rgb) + (size_t)i * kRgbWords;
        uint4 *dr = reinterpret_cast<uint4 *>(sv.vox_rgb) + (size_t)dst * kRgbWords;
        for (int w = threadIdx.x; w < kRgbWords; w += blockDim.x) dr[w] = sr[w];
        if (threadIdx.x == 0) {
            sv.bcoord[dst] = sv.bcoord[i];
            sv.bstamp[dst] = sv.bstamp[i];
            sv.bfresh[dst] = sv.bfresh[i];
        }
    }
}

__global__ void gc_clear_table_kernel(HashSlot *t, int cap) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        HashSlot s;
        s.key = kEmptyKey;
        s.ptr = -1;
        s.pad = 0;
        t[i] = s;
    }
}

// The K kept blocks back into the cleared table (the probe limit of every
// insertion holds: a block that cannot be placed raises GBF_FLAG_HASH_FULL, as
// an allocation would), then the counters.
__global__ void gc_insert_kernel(const SessionView *__restrict__ svs, const int *pre) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    const int K = pre[n];
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < K; id += gridDim.x * blockDim.x) {
        const int4 c = sv.bcoord[id];
        const unsigned long long key = pack_key(c.x, c.y, c.z);
        int slot = home_slot(sv, c.x, c.y, c.z);
        bool placed = false;
        for (int p = 0; p < sv.max_probe && !placed; ++p) {
            HashSlot *e = sv.table + slot;
            if (atomicCAS(&e->key, kEmptyKey, key) == kEmptyKey) {
                e->ptr = id;
                sv.bcoord[id].w = slot;
                placed = true;
            } else {
                slot = (slot + 1 == sv.cap) ? 0 : slot + 1;
            }
        }
        if (!placed) raise_flag(sv, GBF_FLAG_HASH_FULL);
    }
}

// every pool block [0, used) into the cleared table at its own id (a restored snapshot)
__global__ void insert_all_kernel(const SessionView *__restrict__ svs) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
        const int4 c = sv.bcoord[id];
        const unsigned long long key = pack_key(c.x, c.y, c.z);
        int slot = home_slot(sv, c.x, c.y, c.z);
        bool placed = false;
        for (int p = 0; p < sv.max_probe && !placed; ++p) {
            HashSlot *e = sv.table + slot;
            if (atomicCAS(&e->key, kEmptyKey, key) == kEmptyKey) {
                e->ptr = id;
                sv.bcoord[id].w = slot;
                placed = true;
            } else {
                slot = (slot + 1 == sv.cap) ? 0 : slot + 1;
            }
        }
        if (!placed) raise_flag(sv, GBF_FLAG_HASH_FULL);
    }
}

__global__ void gc_finish_kernel(const SessionView *__restrict__ svs, const int *pre) {
    const SessionView &sv = svs[0];
    const int n = used_blocks(sv);
    sv.ctr[C_NUSED] = pre[n];
    sv.ctr[C_NVIS] = 0;
    sv.ctr[C_RENDER] = 0;
}

int grid_for(int items, int per_cta) { return std::max(1, std::min((items + per_cta - 1) / per_cta, 152 * 8)); }

// scan, holes, move, table, counters, after the flags are in mesh_off
void collect(gbf_session *s, cudaStream_t st) {
    const SessionView &v = s->view;
    const int pool = s->cfg.num_blocks;
    gc_scan_kernel<<<1, 1024, 0, st>>>(s->d_view, v.mesh_off);
    gc_holes_kernel<<<grid_for(pool, kGcThreads), kGcThreads, 0, st>>>(s->d_view, v.mesh_off, v.vis);
    const int g = grid_for(pool, 1);
    if (s->cfg.voxel_layout == GBF_VOXEL_REF)
        gc_move_kernel<GBF_VOXEL_REF><<<g, 128, 0, st>>>(s->d_view, v.mesh_off, v.vis);
    else if (s->cfg.voxel_layout == GBF_VOXEL_HALF)
        gc_move_kernel<GBF_VOXEL_HALF><<<g, 128, 0, st>>>(s->d_view, v.mesh_off, v.vis);
    else
        gc_move_kernel<GBF_VOXEL_SNORM><<<g, 128, 0, st>>>(s->d_view, v.mesh_off, v.vis);
    gc_clear_table_kernel<<<grid_for(s->cfg.num_buckets, kGcThreads), kGcThreads, 0, st>>>(v.table, s->cfg.num_buckets);
    gc_insert_kernel<<<grid_for(pool, kGcThreads), kGcThreads, 0, st>>>(s->d_view, v.mesh_off);
    gc_finish_kernel<<<1, 1, 0, st>>>(s->d_view, v.mesh_off);
}

void mark(gbf_session *s, const double center[3], double radius, int drop_unobserved, cudaStream_t st) {
    GcArgs a{};
    a.use_radius = (center && radius >= 0.0) ? 1 : 0;
    a.drop_unobserved = drop_unobserved ? 1 : 0;
    if (a.use_radius) {
        a.cx = center[0];
        a.cy = center[1];
        a.cz = center[2];
        a.r2 = radius * radius;
    }
    a.block_metres = 8.0 * (double)s->cfg.voxel_size;
    const int g = grid_for(s->cfg.num_blocks, kGcThreads / 32);
    int *keep = s->view.mesh_off;
    if (s->cfg.voxel_layout == GBF_VOXEL_REF)
        gc_mark_kernel<GBF_VOXEL_REF><<<g, kGcThreads, 0, st>>>(s->d_view, a, keep);
    else if (s->cfg.voxel_layout == GBF_VOXEL_HALF)
        gc_mark_kernel<GBF_VOXEL_HALF><<<g, kGcThreads, 0, st>>>(s->d_view, a, keep);
    else
        gc_mark_kernel<GBF_VOXEL_SNORM><<<g, kGcThreads, 0, st>>>(s->d_view, a, keep);
}

gbf_status deleted_count(gbf_session *s, cudaStream_t st, int64_t *n_deleted, const char *what) {
    int d = 0;
    cudaError_t e = cudaMemcpyAsync(&d, s->view.ctr + C_GC_DELETED, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, what);
    if (n_deleted) *n_deleted = d;
    return check_cuda(what);
}

}  // namespace

void rebuild_table(gbf_session *s, cudaStream_t st) {
    gc_clear_table_kernel<<<grid_for(s->cfg.num_buckets, kGcThreads), kGcThreads, 0, st>>>(s->view.table,
                                                                                        s->cfg.num_buckets);
    insert_all_kernel<<<grid_for(s->cfg.num_blocks, kGcThreads), kGcThreads, 0, st>>>(s->d_view);
}

}  // namespace gbf

using namespace gbf;

extern "C" {

GBF_API gbf_status gbf_map_delete_blocks(gbf_session *s, const int32_t *coords, int64_t n, int64_t *n_deleted) {
    if (!s || n < 0 || (n > 0 && !coords)) return set_error(GBF_ERR_INVALID_ARG, "gbf_map_delete_blocks: null");
    // the synchronous form: after everything queued on the device, on any stream
    cudaError_t e0 = cudaDeviceSynchronize();
    if (e0 != cudaSuccess) return cuda_error(e0, "gbf_map_delete_blocks");
    cudaStream_t st = nullptr;
    const int pool = s->cfg.num_blocks;
    gc_keep_all_kernel<<<grid_for(pool, kGcThreads), kGcThreads, 0, st>>>(s->d_view, s->view.mesh_off);
    // the list goes through the visible-list array, as many coordinates at a
    // time as its allocation holds
    const int64_t chunk = std::max<int64_t>(1, (int64_t)(s->lay.mesh_off - s->lay.vis) / (3 * sizeof(int32_t)));
    for (int64_t first = 0; first < n; first += chunk) {
        const int m = (int)std::min(chunk, n - first);
        cudaError_t e = cudaMemcpyAsync(s->view.vis, coords + 3 * first, (size_t)m * 3 * sizeof(int32_t),
                                        cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_error(e, "gbf_map_delete_blocks");
        gc_unmark_list_kernel<<<grid_for(m, kGcThreads), kGcThreads, 0, st>>>(s->d_view, s->view.vis, m,
                                                                              s->view.mesh_off);
    }
    collect(s, st);
    return deleted_count(s, st, n_deleted, "gbf_map_delete_blocks");
}

GBF_API gbf_status gbf_map_prune_async(gbf_session *s, const double center[3], double radius,
                                       int32_t drop_unobserved, void *stream) {
    if (!s) return set_error(GBF_ERR_INVALID_ARG, "gbf_map_prune_async: null");
    cudaStream_t st = (cudaStream_t)stream;
    mark(s, center, radius, drop_unobserved, st);
    collect(s, st);
    return check_cuda("gbf_map_prune_async");
}

GBF_API gbf_status gbf_map_prune(gbf_session *s, const double center[3], double radius, int32_t drop_unobserved,
                                 int64_t *n_deleted) {
    if (!s) return set_error(GBF_ERR_INVALID_ARG, "gbf_map_prune: null");
    // the synchronous form: after everything queued on the device, on any stream
    cudaError_t e0 = cudaDeviceSynchronize();
    if (e0 != cudaSuccess) return cuda_error(e0, "gbf_map_prune");
    cudaStream_t st = nullptr;
    mark(s, center, radius, drop_unobserved, st);
    collect(s, st);
    return deleted_count(s, st, n_deleted, "gbf_map_prune");
}

}  // extern "C"
