// mapping.cu -- block allocation, visible-block enumeration and TSDF/colour
// integration (src/voxel_hashing/depth_fusion.cu:15-575 and the hash core of
// src/data_struct/map_struct.cu:143-389).
//
// GB300 design, per frame and for every session of a batch:
//   fuse_begin  bump the session's fuse counter, clear the visible count.
//   alloc       one thread per level-0 pixel walks the blocks of its truncation
//               band (3-D Bresenham, depth_fusion.cu:121-228); the CTA dedupes
//               the keys of its 16x16 pixel tile in a shared-memory set and each
//               unique key is inserted once into the session's open-addressing
//               table with a 64-bit CAS (lock-free, no dropped blocks), stamping
//               the block with the fuse counter.
//   visible     one thread per ALLOCATED block (not per table slot): visible =
//               stamped this fuse OR a block corner projects into the image
//               within [zmin, zmax] (is_block_visible, depth_fusion.cu:15-47);
//               warp-aggregated append to the visible list.
//   integrate   one CTA per visible block (grid-stride), 4 voxels per thread,
//               coalesced SoA voxel read-modify-write; blocks allocated this
//               fuse skip the read and are written whole (lazy zeroing instead
//               of the reference's full-pool cudaMemset, map_struct.cu:90).
#include "gbf_device.cuh"
#include "gbf_kernels.h"

namespace gbf {

namespace {

constexpr int kAllocTile = 16;        // 16x16 pixels per CTA
constexpr int kSetSize = 1024;        // shared-memory key set per CTA

__global__ void fuse_begin_kernel(const SessionView *__restrict__ svs) {
    const SessionView &sv = svs[blockIdx.x];
    if (!sv.active || threadIdx.x != 0) return;
    sv.ctr[C_FRAME] += 1;
    sv.ctr[C_NVIS] = 0;
}

__global__ void fuse_import_kernel(const SessionView *__restrict__ svs, FuseImport in) {
    const SessionView &sv = svs[0];
    const int W = sv.lv[0].w, H = sv.lv[0].h;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    const int x = i % W, y = i / W;
    sv.depth_raw[i] = reinterpret_cast<const float *>(reinterpret_cast<const char *>(in.depth) + y * in.depth_pitch)[x];
    const uint8_t *px = in.rgb + y * in.rgb_pitch + (size_t)x * 3;
    sv.rgb4[i] = make_uchar4(px[0], px[1], px[2], 0);
    if (in.nmap)
        sv.nmap_ext[i] = reinterpret_cast<const float4 *>(reinterpret_cast<const char *>(in.nmap) + y * in.nmap_pitch)[x];
}

// Shared-memory set insert; false when the set is full (caller inserts globally).
__device__ __forceinline__ bool set_insert(unsigned long long *set, unsigned long long key) {
    unsigned h = (unsigned)(key ^ (key >> 29) ^ (key >> 43)) * 0x9E3779B1u;
    unsigned s = h >> (32 - 10);  // kSetSize = 1024
    for (int p = 0; p < 64; ++p) {
        const unsigned long long old = atomicCAS(set + s, kEmptyKey, key);
        if (old == kEmptyKey || old == key) return true;
        s = (s + 1) & (kSetSize - 1);
    }
    return false;
}

__device__ __forceinline__ void visit_block(const SessionView &sv, unsigned long long *set, int bx, int by, int bz,
                                            int frame) {
    if (!coord_ok(bx, by, bz)) {
        raise_flag(sv, GBF_FLAG_COORD_RANGE);
        return;
    }
    const unsigned long long key = pack_key(bx, by, bz);
    if (!set_insert(set, key)) insert_block(sv, key, bx, by, bz, frame);
}

// unproject_world (depth_fusion.cu:101-112) then worldPtToVoxelPos + voxelPosToBlockPos
__device__ __forceinline__ int3 pixel_block(const SessionView &sv, const M34 &T, int x, int y, float z) {
    const LevelK &K = sv.lv[0];
    const float px = (K.invfx * ((float)x - K.cx)) * z;
    const float py = (K.invfy * ((float)y - K.cy)) * z;
    const float3 w = T.apply(px, py, z);
    return make_int3(voxel_to_block(floor_ref(w.x / sv.voxel)), voxel_to_block(floor_ref(w.y / sv.voxel)),
                     voxel_to_block(floor_ref(w.z / sv.voxel)));
}

__global__ void __launch_bounds__(kAllocTile *kAllocTile) alloc_kernel(const SessionView *svs) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    const int W = sv.lv[0].w, H = sv.lv[0].h;
    const int tiles_x = (W + kAllocTile - 1) / kAllocTile;
    const int x = (blockIdx.x % tiles_x) * kAllocTile + (threadIdx.x % kAllocTile);
    const int y = (blockIdx.x / tiles_x) * kAllocTile + (threadIdx.x / kAllocTile);
    if ((blockIdx.x / tiles_x) * kAllocTile >= H) return;  // uniform per CTA

    __shared__ unsigned long long set[kSetSize];
    __shared__ M34 T;
    for (int i = threadIdx.x; i < kSetSize; i += blockDim.x) set[i] = kEmptyKey;
    if (threadIdx.x == 0) T = load_m34(sv.ts->map_twc);
    __syncthreads();
    const int frame = sv.ctr[C_FRAME];

    if (x < W && y < H) {
        const float z = sv.depth_raw[(size_t)y * W + x];
        // create_blocks_kernel (depth_fusion.cu:130-141)
        if (!(isnan(z) || z < sv.zmin_u || z > sv.zmax_u)) {
            const float z_thresh = sv.tau * 0.5f;
            const float z_near = fmaxf(sv.zmin_u, z - z_thresh);
            const float z_far = fminf(sv.zmax_u, z + z_thresh);
            if (z_near < z_far) {
                int3 bn = pixel_block(sv, T, x, y, z_near);
                const int3 bf = pixel_block(sv, T, x, y, z_far);
                const int3 d = make_int3(bf.x - bn.x, bf.y - bn.y, bf.z - bn.z);
                const int3 inc = make_int3(d.x < 0 ? -1 : 1, d.y < 0 ? -1 : 1, d.z < 0 ? -1 : 1);
                const int3 ab = make_int3(abs(d.x), abs(d.y), abs(d.z));
                const int3 e2 = make_int3(ab.x << 1, ab.y << 1, ab.z << 1);
                visit_block(sv, set, bn.x, bn.y, bn.z, frame);
                // Bresenham's line over block coordinates (depth_fusion.cu:153-227)
                if (ab.x >= ab.y && ab.x >= ab.z) {
                    int err1 = e2.y - 1, err2 = e2.z - 1;
                    for (int i = 0; i < ab.x; ++i) {
                        if (err1 > 0) { bn.y += inc.y; err1 -= e2.x; }
                        if (err2 > 0) { bn.z += inc.z; err2 -= e2.x; }
                        err1 += e2.y; err2 += e2.z; bn.x += inc.x;
                        visit_block(sv, set, bn.x, bn.y, bn.z, frame);
                    }
                } else if (ab.y >= ab.x && ab.y >= ab.z) {
                    int err1 = e2.x - 1, err2 = e2.z - 1;
                    for (int i = 0; i < ab.y; ++i) {
                        if (err1 > 0) { bn.x += inc.x; err1 -= e2.y; }
                        if (err2 > 0) { bn.z += inc.z; err2 -= e2.y; }
                        err1 += e2.x; err2 += e2.z; bn.y += inc.y;
                        visit_block(sv, set, bn.x, bn.y, bn.z, frame);
                    }
                } else {
                    int err1 = e2.y - 1, err2 = e2.x - 1;
                    for (int i = 0; i < ab.z; ++i) {
                        if (err1 > 0) { bn.y += inc.y; err1 -= e2.z; }
                        if (err2 > 0) { bn.x += inc.x; err2 -= e2.z; }
                        err1 += e2.y; err2 += e2.x; bn.z += inc.z;
                        visit_block(sv, set, bn.x, bn.y, bn.z, frame);
                    }
                }
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kSetSize; i += blockDim.x) {
        const unsigned long long key = set[i];
        if (key == kEmptyKey) continue;
        // unpack the 21-bit fields (sign-extend)
        const int bx = (int)((long long)(key << (64 - 3 * kCoordBits)) >> (64 - kCoordBits));
        const int by = (int)((long long)(key << (64 - 2 * kCoordBits)) >> (64 - kCoordBits));
        const int bz = (int)((long long)(key << (64 - kCoordBits)) >> (64 - kCoordBits));
        insert_block(sv, key, bx, by, bz, frame);
    }
}

// Per-pixel part of the integration test and weight (update_map_with_colour_kernel,
// depth_fusion.cu:317-331, mode 0; update_map_weighted_kernel, :390-405, mode 2):
// every voxel projecting to a pixel shares them, so they are computed once per
// pixel.  Mode 1 (System frames) gets the same values from level_maps_kernel.
__global__ void fuse_prep_kernel(const SessionView *__restrict__ svs, int mode) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    const int n = sv.lv[0].w * sv.lv[0].h;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float dist = sv.depth_raw[i];
    bool ok;
    float w;
    if (mode == 0) {
        ok = !(isnan(dist) || (double)dist < 1e-2 || dist > sv.zmax_u || dist < sv.zmin_u);
        w = 1.0f / (dist * dist);
    } else {
        const float4 nc = sv.nmap_ext[i];
        ok = !(isnan(dist) || isnan(nc.x) || dist > sv.zmax_u || dist < sv.zmin_u);
        w = fabsf(sinf(nc.z)) / (dist * dist);
    }
    sv.fuse_px[i] = make_float2(ok ? dist : __int_as_float(0x7fffffff), w);
}

// is_vertex_visible / is_block_visible (depth_fusion.cu:15-47)
__device__ __forceinline__ bool block_in_frustum(const SessionView &sv, const M34 &Tcw, int bx, int by, int bz) {
    const LevelK &K = sv.lv[0];
    const float scale = sv.block_metric;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int cx = bx + ((c & 1) ? 1 : 0), cy = by + ((c & 2) ? 1 : 0), cz = bz + ((c & 4) ? 1 : 0);
        const float3 p = Tcw.apply((float)cx * scale, (float)cy * scale, (float)cz * scale);
        const float u = (K.fx * p.x) / p.z + K.cx;
        const float v = (K.fy * p.y) / p.z + K.cy;
        if (!(u < 0 || v < 0 || u > (float)(K.w - 1) || v > (float)(K.h - 1) || p.z < sv.zmin_u || p.z > sv.zmax_u))
            return true;
    }
    return false;
}

__global__ void vis_begin_kernel(const SessionView *__restrict__ svs) {
    const SessionView &sv = svs[blockIdx.x];
    if (!sv.active || threadIdx.x != 0) return;
    sv.ctr[C_NVIS] = 0;
}

// touched: also count blocks stamped by this fuse (check_visibility_flag_kernel's
// flag 2); without it, the frustum test alone (count_visible_entry,
// ray_tracing.cu:778-807 with VisibleEntryEvaluateFunctor, :681-710).
template <bool TOUCHED>
__global__ void __launch_bounds__(256, 6) visible_kernel(const SessionView *svs) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    __shared__ M34 Tcw;
    if (threadIdx.x == 0) Tcw = load_m34(sv.ts->map_tcw);
    __syncthreads();
    const int frame = sv.ctr[C_FRAME];
    const int n = min(sv.ctr[C_NUSED], sv.pool);
    const int stride = gridDim.x * blockDim.x;
    // whole warps iterate together so the append stays warp-uniform
    for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const int id = base + threadIdx.x;
        bool vis = false;
        int tag = 0;
        if (id < n) {
            const int4 c = sv.bcoord[id];
            vis = (TOUCHED && sv.bstamp[id] == frame) || block_in_frustum(sv, Tcw, c.x, c.y, c.z);
            tag = sv.bfresh[id] ? (int)0x80000000 : 0;
        }
        const int pos = warp_append(sv.ctr + C_NVIS, vis);
        if (vis) sv.vis[pos] = id | tag;
    }
}

constexpr int kIntThreads = 128;  // threads per integration CTA (512 / kIntThreads voxels each), 16 CTAs per SM

template <int LAYOUT>
__global__ void __launch_bounds__(kIntThreads, 16) integrate_kernel(const SessionView *__restrict__ svs, int mode) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active || sv.layout != LAYOUT) return;
    __shared__ M34 Tcw_s;
    if (threadIdx.x == 0) Tcw_s = load_m34(sv.ts->map_tcw);
    __syncthreads();
    // Everything the voxel loop reads from the session descriptor is copied to
    // registers first: the loop stores voxels through global pointers, which the
    // compiler would otherwise have to assume may alias the descriptor.
    const M34 Tcw = Tcw_s;
    const LevelK K = sv.lv[0];
    const int W = K.w, H = K.h;
    const int nvis = sv.ctr[C_NVIS];
    if (blockIdx.x == 0 && threadIdx.x == 0) sv.ts->integrated_blocks += nvis;
    const float voxel = sv.voxel, tau = sv.tau, inv_tau = sv.inv_tau;
    const int *__restrict__ vis = sv.vis;
    const int4 *__restrict__ bcoord = sv.bcoord;
    const float2 *__restrict__ fuse_px = sv.fuse_px;
    const uchar4 *__restrict__ rgb4 = sv.rgb4;
    unsigned char *__restrict__ bfresh = sv.bfresh;
    void *__restrict__ vox_sw = sv.vox_sw;
    uchar4 *__restrict__ vox_rgb = sv.vox_rgb;

    for (int b = blockIdx.x; b < nvis; b += gridDim.x) {
        const int tagged = vis[b];
        const int id = tagged & 0x7fffffff;
        const bool fresh = tagged < 0;
        const int4 bc = bcoord[id];
#pragma unroll
        for (int half_i = 0; half_i < kBlockVoxels / kIntThreads; ++half_i) {
            const int li = threadIdx.x + half_i * kIntThreads;
            const int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
            const int vi = id * kBlockVoxels + li;
            const float3 p = Tcw.apply((float)(bc.x * 8 + lx) * voxel, (float)(bc.y * 8 + ly) * voxel,
                                       (float)(bc.z * 8 + lz) * voxel);
            const int u = __float2int_rd(((K.fx * p.x) / p.z + K.cx) + 0.5f);
            const int v = __float2int_rd(((K.fy * p.y) / p.z + K.cy) + 0.5f);
            bool upd = !(u < 0 || v < 0 || u > W - 1 || v > H - 1);
            float dist = 0.f, weight = 0.f, sdf = 0.f;
            if (upd) {
                // depth and weight of the pixel, rejected pixels as NaN (fuse_px)
                const float2 fp = fuse_px[v * W + u];
                dist = fp.x;
                weight = fp.y;
                upd = !isnan(dist);
            }
            if (upd) {
                sdf = dist - p.z;
                if (sdf < -tau) upd = false;
            }
            if (!upd) {
                if (fresh) {
                    store_sw_at<LAYOUT>(vox_sw, vi, 0.f, 0.f);
                    vox_rgb[vi] = make_uchar4(0, 0, 0, 0);
                }
                continue;
            }
            sdf = fminf(1.0f, sdf * inv_tau);
            Vox old;
            if (fresh) {
                old.sdf = 0.f; old.w = 0.f; old.rgb = make_uchar4(0, 0, 0, 0);
            } else {
                old = load_vox_at<LAYOUT>(vox_sw, vox_rgb, vi);
            }
            const uchar4 cn = rgb4[v * W + u];
            float nsdf, nw;
            uchar4 nrgb;
            if (old.w == 0.f) {
                nsdf = sdf; nw = weight; nrgb = cn;
            } else {
                // the four running means share one denominator: one correctly
                // rounded reciprocal, then each quotient by div_rn_by
                const float den = old.w + weight;
                const float rden = __frcp_rn(den);
                nsdf = div_rn_by(old.sdf * old.w + sdf * weight, den, rden);
                nw = old.w + weight;
                nrgb.x = (unsigned char)__float2int_rz(
                    div_rn_by((float)old.rgb.x * old.w + (float)cn.x * weight, den, rden));
                nrgb.y = (unsigned char)__float2int_rz(
                    div_rn_by((float)old.rgb.y * old.w + (float)cn.y * weight, den, rden));
                nrgb.z = (unsigned char)__float2int_rz(
                    div_rn_by((float)old.rgb.z * old.w + (float)cn.z * weight, den, rden));
                nrgb.w = 0;
            }
            store_sw_at<LAYOUT>(vox_sw, vi, nsdf, nw);
            vox_rgb[vi] = nrgb;
        }
        if (fresh && threadIdx.x == 0) bfresh[id] = 0;
    }
}

}  // namespace

void launch_fuse_import(const SessionView *d_sv, const Extent &ex, const FuseImport &in, cudaStream_t st) {
    const int n = ex.w * ex.h;
    fuse_import_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_sv, in);
}

// CTAs per session of the visible-block pass (grid-stride over the allocated
// blocks, whose count only the device knows); enough for a pool's worth
// without launching a CTA per 256 pool slots
constexpr int kVisCtas = 152;

void launch_alloc_visible(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st) {
    fuse_begin_kernel<<<nslots, 32, 0, st>>>(d_sv);
    const int tiles = ((ex.w + kAllocTile - 1) / kAllocTile) * ((ex.h + kAllocTile - 1) / kAllocTile);
    alloc_kernel<<<dim3(tiles, nslots), kAllocTile * kAllocTile, 0, st>>>(d_sv);
    const int gv = min(max((ex.max_pool + 255) / 256, 1), kVisCtas);
    visible_kernel<true><<<dim3(gv, nslots), 256, 0, st>>>(d_sv);
}

void launch_visible_frustum(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st) {
    vis_begin_kernel<<<nslots, 32, 0, st>>>(d_sv);
    const int gv = min(max((ex.max_pool + 255) / 256, 1), kVisCtas);
    visible_kernel<false><<<dim3(gv, nslots), 256, 0, st>>>(d_sv);
}

void launch_integrate(const SessionView *d_sv, int nslots, const Extent &ex, int mode, const int *layouts,
                      cudaStream_t st) {
    if (mode != 1) fuse_prep_kernel<<<dim3((ex.w * ex.h + 255) / 256, nslots), 256, 0, st>>>(d_sv, mode);
    // one CTA per visible block, grid-stride over 8 CTAs per SM per session (16 of
    // 128 threads are resident per SM)
    const int gi = 152 * 8;
    if (layouts[GBF_VOXEL_REF]) integrate_kernel<GBF_VOXEL_REF><<<dim3(gi, nslots), kIntThreads, 0, st>>>(d_sv, mode);
    if (layouts[GBF_VOXEL_HALF]) integrate_kernel<GBF_VOXEL_HALF><<<dim3(gi, nslots), kIntThreads, 0, st>>>(d_sv, mode);
    if (layouts[GBF_VOXEL_SNORM]) integrate_kernel<GBF_VOXEL_SNORM><<<dim3(gi, nslots), kIntThreads, 0, st>>>(d_sv, mode);
}

void launch_fuse(const SessionView *d_sv, int nslots, const Extent &ex, int mode, const int *layouts,
                 cudaStream_t st) {
    launch_alloc_visible(d_sv, nslots, ex, st);
    launch_integrate(d_sv, nslots, ex, mode, layouts, st);
}

}  // namespace gbf
