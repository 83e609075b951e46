// raycast.cu -- z-range tiles and per-pixel raycast (src/voxel_hashing/
// ray_tracing.cu:63-425) plus the post-raycast pyramid (DeviceImage::
// resize_device_map, src/tracking/device_image.cpp:188-199).
//
// GB300 design:
//   zr_init   z-range grid (H/8 x W/8) to (100, 0), render counter to 0.
//   zrange    one thread per visible block: the block's screen box on the 1/8
//             grid and its depth interval (create_rendering_block, :63-126), then
//             integer atomicMin / atomicMax on the float bit patterns (all values
//             are positive) of every covered cell.  The reference's 16x16
//             rendering-tile list, its cudaMalloc and its host read-back
//             (:223-277) are gone; the union of its tiles is exactly the box.
//   raycast   one thread per pixel, 64-pixel CTAs (8x8 by default: a warp is
//             an 8x4 patch);
//             the march of MapRenderingDelegate::operator() (:346-425) with a
//             per-thread cache of the last block lookup, so trilinear samples
//             within one block cost one hash probe; a trilinear read spanning
//             blocks looks each block up once, out of line.  Output:
//             camera-frame float4 vertex (NaN = miss).
//   post      2x2 mean vertex pyramid, then normals of every level.
#include "gbf_device.cuh"
#include "gbf_kernels.h"

namespace gbf {

namespace {

__global__ void zr_init_kernel(const SessionView *__restrict__ svs) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    const int n = sv.zr_w * sv.zr_h;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        sv.zr_min[i] = 100.f;
        sv.zr_max[i] = 0.f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sv.ctr[C_RENDER] = 0;
}

__global__ void __launch_bounds__(256, 6) zrange_kernel(const SessionView *__restrict__ svs) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    __shared__ M34 Tcw;
    if (threadIdx.x == 0) Tcw = load_m34(sv.ts->map_tcw);
    __syncthreads();
    const int nvis = sv.ctr[C_NVIS];
    const LevelK &K = sv.lv[0];
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nvis; b += gridDim.x * blockDim.x) {
        const int id = sv.vis[b] & 0x7fffffff;
        const int4 bc = sv.bcoord[id];
        int ulx = sv.zr_w, uly = sv.zr_h, lrx = -1, lry = -1;
        float zx = sv.zmax_r, zy = sv.zmin_r;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int cx = bc.x + ((c & 1) ? 1 : 0), cy = bc.y + ((c & 2) ? 1 : 0), cz = bc.z + ((c & 4) ? 1 : 0);
            const float3 p = Tcw.apply((float)cx * sv.block_metric, (float)cy * sv.block_metric,
                                       (float)cz * sv.block_metric);
            const float u = ((K.fx * p.x) / p.z + K.cx) / 8.0f;
            const float v = ((K.fy * p.y) / p.z + K.cy) / 8.0f;
            const float fu = floorf(u), fv = floorf(v), cu = ceilf(u), cv = ceilf(v);
            if ((float)ulx > fu) ulx = __float2int_rz(fu);
            if ((float)lrx < cu) lrx = __float2int_rz(cu);
            if ((float)uly > fv) uly = __float2int_rz(fv);
            if ((float)lry < cv) lry = __float2int_rz(cv);
            if (zx > p.z) zx = p.z;
            if (zy < p.z) zy = p.z;
        }
        if (ulx < 0) ulx = 0;
        if (uly < 0) uly = 0;
        if (lrx >= sv.zr_w) lrx = sv.zr_w - 1;
        if (lry >= sv.zr_h) lry = sv.zr_h - 1;
        if (ulx > lrx || uly > lry) continue;
        if (zx < sv.zmin_r) zx = sv.zmin_r;
        if (zy < sv.zmin_r) continue;
        atomicAdd(sv.ctr + C_RENDER, 1);
        const int ix = __float_as_int(zx), iy = __float_as_int(zy);
        for (int y = uly; y <= lry; ++y)
            for (int x = ulx; x <= lrx; ++x) {
                atomicMin(reinterpret_cast<int *>(sv.zr_min) + y * sv.zr_w + x, ix);
                atomicMax(reinterpret_cast<int *>(sv.zr_max) + y * sv.zr_w + x, iy);
            }
    }
}

// Last block lookup of a ray: consecutive samples usually stay in one block.
// (A per-CTA shared-memory cache of block ids in front of the table measured
// slower than going to the table directly.)
struct BlockCache {
    int bx, by, bz, id;
    __device__ __forceinline__ void init() {
        bx = by = bz = 0x7fffffff;
        id = -1;
    }
    template <class SV>
    __device__ __forceinline__ int get(const SV &sv, int x, int y, int z) {
        if (x != bx || y != by || z != bz) {
            bx = x; by = y; bz = z;
            id = find_block(sv, x, y, z);
        }
        return id;
    }
};

// sdf of pool voxel i (int32 index: the pool is validated to fit), or NaN when
// unobserved (weight 0).  Only the weight's zero test is needed, so the HALF
// and SNORM layouts test the binary16 weight bits instead of converting them.
template <int LAYOUT, class SV>
__device__ __forceinline__ float sdf_at(const SV &sv, int i, bool &valid) {
    const float qnan = __int_as_float(0x7fffffff);
    if (LAYOUT == GBF_VOXEL_REF) {
        const uint2 q = __ldg(reinterpret_cast<const uint2 *>(sv.vox_sw) + i);
        valid = __uint_as_float(q.y) != 0.f;
        return valid ? sdf_ref_unpack((short)(q.x & 0xffffu)) : qnan;
    } else {
        const unsigned q = __ldg(reinterpret_cast<const unsigned *>(sv.vox_sw) + i);
        valid = (q & 0x7fff0000u) != 0u;  // binary16 weight != +-0 (NaN counts as observed, as w != 0.f)
        return valid ? sdf_word_unpack<LAYOUT>((unsigned short)(q & 0xffffu)) : qnan;
    }
}

// One voxel by integer position: sdf, or NaN when unallocated or unobserved.
template <int LAYOUT, class SV>
__device__ __forceinline__ float read_vox(const SV &sv, BlockCache &bc, int vx, int vy, int vz,
                                          bool &valid) {
    const int id = bc.get(sv, voxel_to_block(vx), voxel_to_block(vy), voxel_to_block(vz));
    if (id >= 0)
        return sdf_at<LAYOUT>(sv, id * kBlockVoxels + (voxel_to_local(vz) * 64 + voxel_to_local(vy) * 8 +
                                                       voxel_to_local(vx)), valid);
    valid = false;
    return __int_as_float(0x7fffffff);
}

// Voxel (vx, vy, vz) of block id (looked up by the caller): sdf, or NaN when
// the block is unallocated (id < 0) or the voxel unobserved.
template <int LAYOUT, class SV>
__device__ __forceinline__ float vox_in(const SV &sv, int id, int vx, int vy, int vz, bool &valid) {
    if (id >= 0)
        return sdf_at<LAYOUT>(sv, id * kBlockVoxels + (voxel_to_local(vz) * 64 + voxel_to_local(vy) * 8 +
                                                       voxel_to_local(vx)), valid);
    valid = false;
    return __int_as_float(0x7fffffff);
}

// read_sdf (ray_tracing.cu:291-305): nearest voxel ToVector3i(pt)
template <int LAYOUT, class SV>
__device__ __forceinline__ float read_sdf(const SV &sv, BlockCache &bc, float px, float py, float pz,
                                          bool &valid) {
    return read_vox<LAYOUT>(sv, bc, floor_ref(px), floor_ref(py), floor_ref(pz), valid);
}

// The trilinear read when the corners span two to eight blocks (about 1/3 of
// the reads): out of line, so that the march loop's code stays small.  i000:
// the block of corner (x0, y0, z0), looked up by the caller.
template <int LAYOUT, class SV>
__device__ __noinline__ float interp_spanning(const SV sv, int i000, int x0, int x1, int y0, int y1, int z0, int z1,
                                              float fx, float fy, float fz, float s000, bool v000, bool have000,
                                              bool &valid) {
    const int bx0 = voxel_to_block(x0), bx1 = voxel_to_block(x1), by0 = voxel_to_block(y0),
              by1 = voxel_to_block(y1), bz0 = voxel_to_block(z0), bz1 = voxel_to_block(z1);
    const bool sx = bx1 != bx0, sy = by1 != by0, sz = bz1 != bz0;
    const int i100 = sx ? find_block(sv, bx1, by0, bz0) : i000;
    const int i010 = sy ? find_block(sv, bx0, by1, bz0) : i000;
    const int i110 = (sx && sy) ? find_block(sv, bx1, by1, bz0) : (sx ? i100 : i010);
    const int i001 = sz ? find_block(sv, bx0, by0, bz1) : i000;
    const int i101 = sz ? (sx ? find_block(sv, bx1, by0, bz1) : i001) : i100;
    const int i011 = sz ? (sy ? find_block(sv, bx0, by1, bz1) : i001) : i010;
    const int i111 = sz ? ((sx && sy) ? find_block(sv, bx1, by1, bz1) : (sx ? i101 : i011)) : i110;
    bool vpt, v;
    float s0, s1, r0, r1, r2, r3;
    if (have000) {
        s0 = s000;
        vpt = v000;
    } else {
        s0 = vox_in<LAYOUT>(sv, i000, x0, y0, z0, vpt);
    }
    s1 = vox_in<LAYOUT>(sv, i100, x1, y0, z0, v);
    vpt &= v;
    r0 = (1.0f - fx) * s0 + fx * s1;
    s0 = vox_in<LAYOUT>(sv, i010, x0, y1, z0, v);
    vpt &= v;
    s1 = vox_in<LAYOUT>(sv, i110, x1, y1, z0, v);
    vpt &= v;
    r1 = (1.0f - fx) * s0 + fx * s1;
    r2 = (1.0f - fy) * r0 + fy * r1;
    s0 = vox_in<LAYOUT>(sv, i001, x0, y0, z1, v);
    vpt &= v;
    s1 = vox_in<LAYOUT>(sv, i101, x1, y0, z1, v);
    vpt &= v;
    r0 = (1.0f - fx) * s0 + fx * s1;
    s0 = vox_in<LAYOUT>(sv, i011, x0, y1, z1, v);
    vpt &= v;
    s1 = vox_in<LAYOUT>(sv, i111, x1, y1, z1, v);
    vpt &= v;
    r1 = (1.0f - fx) * s0 + fx * s1;
    r3 = (1.0f - fy) * r0 + fy * r1;
    valid = vpt;
    return (1.0f - fz) * r2 + fz * r3;
}


// read_sdf_interped (ray_tracing.cu:307-339).  The reference reads the eight
// corners at pt + (0|1, 0|1, 0|1) and floors each sum; the six per-axis floors
// floor(p), floor(p + 1) are computed once (floor(p + 1) is not always
// floor(p) + 1 in float).  s000 / v000: the corner at floor(pt) when the caller
// has already read it.  When the eight corners lie in one block (about 2/3 of
// the samples) they are read by offset from one lookup, all loads issued
// together; the arithmetic is the same in both paths.
template <int LAYOUT, bool HAVE000, class SV>
__device__ __forceinline__ float read_sdf_interped(const SV &sv, BlockCache &bc, float px, float py,
                                                   float pz, bool &valid, float s000 = 0.f, bool v000 = false) {
    const float fx = px - floorf(px), fy = py - floorf(py), fz = pz - floorf(pz);
    const int x0 = floor_ref(px + 0.0f), x1 = floor_ref(px + 1.0f);
    const int y0 = floor_ref(py + 0.0f), y1 = floor_ref(py + 1.0f);
    const int z0 = floor_ref(pz + 0.0f), z1 = floor_ref(pz + 1.0f);
    bool vpt;
    float r0, r1, r2, r3;
    if (x1 == x0 + 1 && y1 == y0 + 1 && z1 == z0 + 1 && (x0 & 7) != 7 && (y0 & 7) != 7 && (z0 & 7) != 7) {
        const int id = bc.get(sv, voxel_to_block(x0), voxel_to_block(y0), voxel_to_block(z0));
        if (id < 0) {  // every corner unallocated: the general path's NaN arithmetic, invalid
            valid = false;
            return __int_as_float(0x7fffffff);
        }
        const int i = id * kBlockVoxels + (voxel_to_local(z0) * 64 + voxel_to_local(y0) * 8 + voxel_to_local(x0));
        bool v1, v2, v3, v4, v5, v6, v7;
        float c000;
        if (HAVE000) {
            c000 = s000;
            vpt = v000;
        } else {
            c000 = sdf_at<LAYOUT>(sv, i, vpt);
        }
        const float c100 = sdf_at<LAYOUT>(sv, i + 1, v1), c010 = sdf_at<LAYOUT>(sv, i + 8, v2);
        const float c110 = sdf_at<LAYOUT>(sv, i + 9, v3), c001 = sdf_at<LAYOUT>(sv, i + 64, v4);
        const float c101 = sdf_at<LAYOUT>(sv, i + 65, v5), c011 = sdf_at<LAYOUT>(sv, i + 72, v6);
        const float c111 = sdf_at<LAYOUT>(sv, i + 73, v7);
        r0 = (1.0f - fx) * c000 + fx * c100;
        r1 = (1.0f - fx) * c010 + fx * c110;
        r2 = (1.0f - fy) * r0 + fy * r1;
        r0 = (1.0f - fx) * c001 + fx * c101;
        r1 = (1.0f - fx) * c011 + fx * c111;
        r3 = (1.0f - fy) * r0 + fy * r1;
        valid = vpt && v1 && v2 && v3 && v4 && v5 && v6 && v7;
        return (1.0f - fz) * r2 + fz * r3;
    }
    const int i000 = bc.get(sv, voxel_to_block(x0), voxel_to_block(y0), voxel_to_block(z0));
    return interp_spanning<LAYOUT>(sv, i000, x0, x1, y0, y1, z0, z1, fx, fy, fz, s000, v000, HAVE000, valid);
}

// The fields the march reads on every step, copied into registers once per
// thread: through the descriptor in global memory the compiler has to reload
// them (the same copy took the integration from 2.29 to 1.76 ms).
struct MarchView {
    const HashSlot *table;
    void *vox_sw;
    int cap, cap_mask, max_probe;
};

// One CTA marches a tile of kRayThreads pixels, tw wide and kRayThreads / tw
// high (tw = 4, 8, 16 or 32; the launch shape is a batch knob).  The default
// 8x8 tile gives each warp an 8x4 patch: coherent march lengths.
constexpr int kRayThreads = 64;
constexpr int kMaxMarch = 1 << 16;  // safety bound; the march advances >= 1 voxel per step

// RGB: also write the hits' voxel colours (a separate instantiation: the
// colour pointer kept live across the march costs the plain raycast spills).
template <int LAYOUT, bool RGB>
__global__ void __launch_bounds__(kRayThreads, 24) raycast_kernel(const SessionView *__restrict__ svs, float4 *vmap_ext,
                                                                  long long vmap_pitch, int tw, uint8_t *rgb_ext,
                                                                  long long rgb_pitch) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active || sv.layout != LAYOUT) return;
    // the reference skips the raycast when nothing was visible or renderable
    if (sv.ctr[C_NVIS] == 0 || sv.ctr[C_RENDER] == 0) return;
    const LevelK &K = sv.lv[0];
    const int th = kRayThreads / tw;
    const int tiles_x = (K.w + tw - 1) / tw;
    const int x = (blockIdx.x % tiles_x) * tw + (threadIdx.x % tw);
    const int y = (blockIdx.x / tiles_x) * th + (threadIdx.x / tw);
    __shared__ M34 Twc, Tcw;
    if (threadIdx.x == 0) {
        Tcw = load_m34(sv.ts->map_tcw);
        Twc = load_m34(sv.ts->map_twc);
    }
    __syncthreads();
    if (x >= K.w || y >= K.h) return;

    float4 *out = vmap_ext ? reinterpret_cast<float4 *>(reinterpret_cast<char *>(vmap_ext) + y * vmap_pitch) + x
                           : sv.vmap[sv.ts->idx][0] + (size_t)y * K.w + x;
    const float qnan = __int_as_float(0x7fffffff);
    *out = make_float4(qnan, qnan, qnan, qnan);
    // colour (raycast_with_colour, ray_tracing.cu:478-564): white unless a hit's
    // nearest voxel has been observed
    if (RGB) {
        uint8_t *px = rgb_ext + y * rgb_pitch + (long long)x * 3;
        px[0] = px[1] = px[2] = 255;
    }

    const int cx = __float2int_rd((float)x / 8), cy = __float2int_rd((float)y / 8);
    if (cx >= sv.zr_w || cy >= sv.zr_h) return;
    const float zr0 = sv.zr_min[cy * sv.zr_w + cx], zr1 = sv.zr_max[cy * sv.zr_w + cx];
    if ((double)zr1 < 1e-3 || (double)zr0 < 1e-3 || isnan(zr0) || isnan(zr1)) return;

    const float iv = sv.inv_voxel;
    // unproject (ray_tracing.cu:341-344): (x - cx) * invfx * z
    float ux = (((float)x - K.cx) * K.invfx) * zr0, uy = (((float)y - K.cy) * K.invfy) * zr0;
    float dist_s = norm3(ux, uy, zr0) * iv;
    float3 bs = Twc.apply(ux, uy, zr0);
    bs = make_float3(bs.x * iv, bs.y * iv, bs.z * iv);
    ux = (((float)x - K.cx) * K.invfx) * zr1;
    uy = (((float)y - K.cy) * K.invfy) * zr1;
    const float dist_e = norm3(ux, uy, zr1) * iv;
    float3 be = Twc.apply(ux, uy, zr1);
    be = make_float3(be.x * iv, be.y * iv, be.z * iv);
    float3 dir = make_float3(be.x - bs.x, be.y - bs.y, be.z - bs.z);
    const float dn = norm3(dir.x, dir.y, dir.z);
    dir = make_float3(dir.x / dn, dir.y / dn, dir.z / dn);
    float3 r = bs;

    const MarchView mv{sv.table, sv.vox_sw, sv.cap, sv.cap_mask, sv.max_probe};
    const float step_scale = sv.step_scale;
    BlockCache bc;
    bc.init();
    float sdf = 1.0f, last_sdf, step;
    bool valid = false;
    for (int it = 0; dist_s < dist_e && it < kMaxMarch; ++it) {
        last_sdf = sdf;
        sdf = read_sdf<LAYOUT>(mv, bc, r.x, r.y, r.z, valid);
        if (sdf <= 0.5f && sdf >= -0.5f) sdf = read_sdf_interped<LAYOUT, true>(mv, bc, r.x, r.y, r.z, valid, sdf, valid);
        if (sdf <= 0.0f) break;
        if (sdf >= 0.f && last_sdf < 0.f) return;
        step = valid ? fmaxf(sdf * step_scale, 1.0f) : 2.0f;
        r = make_float3(r.x + dir.x * step, r.y + dir.y * step, r.z + dir.z * step);
        dist_s += step;
    }
    bool found = false;
    if (sdf <= 0.0f) {
        step = sdf * step_scale;
        r = make_float3(r.x + dir.x * step, r.y + dir.y * step, r.z + dir.z * step);
        sdf = read_sdf_interped<LAYOUT, false>(mv, bc, r.x, r.y, r.z, valid);
        step = sdf * step_scale;
        r = make_float3(r.x + dir.x * step, r.y + dir.y * step, r.z + dir.z * step);
        found = valid;
    }
    if (found) {
        const float3 c = Tcw.apply(r.x * sv.voxel, r.y * sv.voxel, r.z * sv.voxel);
        *out = make_float4(c.x, c.y, c.z, 1.0f);
        if (RGB) {  // read_colour (ray_tracing.cu:427-441): the voxel ToVector3i(pt)
            const int vx = floor_ref(r.x), vy = floor_ref(r.y), vz = floor_ref(r.z);
            const int id = bc.get(mv, voxel_to_block(vx), voxel_to_block(vy), voxel_to_block(vz));
            if (id >= 0) {
                const int i = id * kBlockVoxels + (voxel_to_local(vz) * 64 + voxel_to_local(vy) * 8 + voxel_to_local(vx));
                bool observed;
                sdf_at<LAYOUT>(mv, i, observed);
                if (observed) {
                    const uchar4 col = sv.vox_rgb[i];
                    uint8_t *px = rgb_ext + y * rgb_pitch + (long long)x * 3;
                    px[0] = col.x;
                    px[1] = col.y;
                    px[2] = col.z;
                }
            }
        }
    }
}

// cv::cuda::resize(vmap, 0.5): 2x2 mean of every channel
__global__ void vmap_down_kernel(const SessionView *__restrict__ svs, int level) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active || level >= sv.levels) return;
    const int w = sv.lv[level].w, h = sv.lv[level].h, pw = sv.lv[level - 1].w;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const int x = i % w, y = i / w;
    const int set = sv.ts->idx;
    const float4 *s = sv.vmap[set][level - 1];
    const float4 a = s[(size_t)(2 * y) * pw + 2 * x], b = s[(size_t)(2 * y) * pw + 2 * x + 1];
    const float4 c = s[(size_t)(2 * y + 1) * pw + 2 * x], d = s[(size_t)(2 * y + 1) * pw + 2 * x + 1];
    sv.vmap[set][level][i] = make_float4((((a.x + b.x) + c.x) + d.x) * 0.25f, (((a.y + b.y) + c.y) + d.y) * 0.25f,
                                         (((a.z + b.z) + c.z) + d.z) * 0.25f, (((a.w + b.w) + c.w) + d.w) * 0.25f);
}

// computeNMapK (cuda_imgproc.cu:276-294) over every level of the reference set
// computeNMapK (cuda_imgproc.cu:276-305) at (x, y) of a vertex map whose rows are
// `stride` float4 apart: normalised cross product of the horizontal and vertical
// differences; NaN in the last row and column (written, where the reference
// leaves them unwritten) and wherever a neighbour is NaN.
template <class Get>
__device__ __forceinline__ float4 normal_by(const Get &V, int x, int y, int w, int h) {
    const float qnan = __int_as_float(0x7fffffff);
    if (x >= w - 1 || y >= h - 1) return make_float4(qnan, qnan, qnan, qnan);
    const int x10 = max(x - 1, 0), y10 = max(y - 1, 0);
    const float4 v00 = V(x10, y), v01 = V(x + 1, y);
    const float4 v10 = V(x, y10), v11 = V(x, y + 1);
    const float3 a = make_float3(v01.x - v00.x, v01.y - v00.y, v01.z - v00.z);
    const float3 bb = make_float3(v11.x - v10.x, v11.y - v10.y, v11.z - v10.z);
    const float3 n = cross3(a, bb);
    const float l = norm3(n.x, n.y, n.z);
    return make_float4(n.x / l, n.y / l, n.z / l, 1.f);
}
__device__ __forceinline__ float4 normal_at(const float4 *V, long long stride, int x, int y, int w, int h) {
    return normal_by([&](int xx, int yy) { return V[yy * stride + xx]; }, x, y, w, h);
}

// 2x2 mean of four vertices in vmap_down_kernel's order
__device__ __forceinline__ float4 mean4(const float4 a, const float4 b, const float4 c, const float4 d) {
    return make_float4((((a.x + b.x) + c.x) + d.x) * 0.25f, (((a.y + b.y) + c.y) + d.y) * 0.25f,
                       (((a.z + b.z) + c.z) + d.z) * 0.25f, (((a.w + b.w) + c.w) + d.w) * 0.25f);
}

// The post-raycast pyramid of up to three levels in one pass: a CTA takes a
// 32x32 tile of the level-0 vertex map with a 4-pixel halo into shared memory,
// writes the tile's level-0 normals, builds the 16x16 level-1 tile (2x2 means,
// vmap_down_kernel's arithmetic) with a 2-pixel halo and its normals, then the
// 8x8 level-2 tile with a 1-pixel halo and its normals -- the arithmetic of
// vmap_down_kernel and nmap_all_kernel, reading the level-0 map once instead of
// writing and re-reading every level.
constexpr int kPostTile = 32;
__global__ void __launch_bounds__(256) post_pyramid_kernel(const SessionView *__restrict__ svs) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    const int w0 = sv.lv[0].w, h0 = sv.lv[0].h;
    const int tiles_x = (w0 + kPostTile - 1) / kPostTile;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    if (ty * kPostTile >= h0) return;  // a smaller frame than the batch's largest
    const int set = sv.ts->idx;
    const float qnan = __int_as_float(0x7fffffff);
    const float4 nan4 = make_float4(qnan, qnan, qnan, qnan);
    __shared__ float4 s0[kPostTile + 8][kPostTile + 8];
    __shared__ float4 s1[kPostTile / 2 + 4][kPostTile / 2 + 4];
    __shared__ float4 s2[kPostTile / 4 + 2][kPostTile / 4 + 2];
    // level 0: the tile and its 4-pixel halo (outside the image: never read)
    const int ox0 = tx * kPostTile - 4, oy0 = ty * kPostTile - 4;
    const float4 *V0 = sv.vmap[set][0];
    for (int i = threadIdx.x; i < (kPostTile + 8) * (kPostTile + 8); i += blockDim.x) {
        const int lx = i % (kPostTile + 8), ly = i / (kPostTile + 8), x = ox0 + lx, y = oy0 + ly;
        s0[ly][lx] = (x >= 0 && y >= 0 && x < w0 && y < h0) ? V0[(size_t)y * w0 + x] : nan4;
    }
    __syncthreads();
    {
        const auto get0 = [&](int x, int y) { return s0[y - oy0][x - ox0]; };
        float4 *N0 = sv.nmap[set][0];
        for (int i = threadIdx.x; i < kPostTile * kPostTile; i += blockDim.x) {
            const int x = tx * kPostTile + i % kPostTile, y = ty * kPostTile + i / kPostTile;
            if (x < w0 && y < h0) N0[(size_t)y * w0 + x] = normal_by(get0, x, y, w0, h0);
        }
    }
    if (sv.levels < 2) return;
    // level 1: the 16x16 tile and a 2-pixel halo, from the level-0 pixels in s0
    const int w1 = sv.lv[1].w, h1 = sv.lv[1].h;
    const int ox1 = tx * (kPostTile / 2) - 2, oy1 = ty * (kPostTile / 2) - 2;
    float4 *V1 = sv.vmap[set][1];
    for (int i = threadIdx.x; i < (kPostTile / 2 + 4) * (kPostTile / 2 + 4); i += blockDim.x) {
        const int lx = i % (kPostTile / 2 + 4), ly = i / (kPostTile / 2 + 4), x = ox1 + lx, y = oy1 + ly;
        float4 v = nan4;
        if (x >= 0 && y >= 0 && x < w1 && y < h1) {
            // level-0 pixel (2x, 2y) sits at s0[2 ly][2 lx]
            v = mean4(s0[2 * ly][2 * lx], s0[2 * ly][2 * lx + 1], s0[2 * ly + 1][2 * lx], s0[2 * ly + 1][2 * lx + 1]);
            if (lx >= 2 && ly >= 2 && lx < kPostTile / 2 + 2 && ly < kPostTile / 2 + 2) V1[(size_t)y * w1 + x] = v;
        }
        s1[ly][lx] = v;
    }
    __syncthreads();
    {
        const auto get1 = [&](int x, int y) { return s1[y - oy1][x - ox1]; };
        float4 *N1 = sv.nmap[set][1];
        for (int i = threadIdx.x; i < (kPostTile / 2) * (kPostTile / 2); i += blockDim.x) {
            const int x = tx * (kPostTile / 2) + i % (kPostTile / 2), y = ty * (kPostTile / 2) + i / (kPostTile / 2);
            if (x < w1 && y < h1) N1[(size_t)y * w1 + x] = normal_by(get1, x, y, w1, h1);
        }
    }
    if (sv.levels < 3) return;
    // level 2: the 8x8 tile and a 1-pixel halo, from the level-1 pixels in s1
    const int w2 = sv.lv[2].w, h2 = sv.lv[2].h;
    const int ox2 = tx * (kPostTile / 4) - 1, oy2 = ty * (kPostTile / 4) - 1;
    float4 *V2 = sv.vmap[set][2];
    for (int i = threadIdx.x; i < (kPostTile / 4 + 2) * (kPostTile / 4 + 2); i += blockDim.x) {
        const int lx = i % (kPostTile / 4 + 2), ly = i / (kPostTile / 4 + 2), x = ox2 + lx, y = oy2 + ly;
        float4 v = nan4;
        if (x >= 0 && y >= 0 && x < w2 && y < h2) {
            // level-1 pixel (2x, 2y) sits at s1[2 ly][2 lx]
            v = mean4(s1[2 * ly][2 * lx], s1[2 * ly][2 * lx + 1], s1[2 * ly + 1][2 * lx], s1[2 * ly + 1][2 * lx + 1]);
            if (lx >= 1 && ly >= 1 && lx < kPostTile / 4 + 1 && ly < kPostTile / 4 + 1) V2[(size_t)y * w2 + x] = v;
        }
        s2[ly][lx] = v;
    }
    __syncthreads();
    const auto get2 = [&](int x, int y) { return s2[y - oy2][x - ox2]; };
    float4 *N2 = sv.nmap[set][2];
    for (int i = threadIdx.x; i < (kPostTile / 4) * (kPostTile / 4); i += blockDim.x) {
        const int x = tx * (kPostTile / 4) + i % (kPostTile / 4), y = ty * (kPostTile / 4) + i / (kPostTile / 4);
        if (x < w2 && y < h2) N2[(size_t)y * w2 + x] = normal_by(get2, x, y, w2, h2);
    }
}

__global__ void nmap_of_kernel(const float4 *vmap, long long vmap_pitch, float4 *nmap, long long nmap_pitch, int w,
                               int h) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    // the pitches are multiples of 16 bytes (checked by the caller)
    reinterpret_cast<float4 *>(reinterpret_cast<char *>(nmap) + y * nmap_pitch)[x] =
        normal_at(vmap, vmap_pitch / 16, x, y, w, h);
}

__global__ void nmap_all_kernel(const SessionView *__restrict__ svs) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    int b = blockIdx.x, level = 0;
    for (; level < sv.levels; ++level) {
        const int n = (sv.lv[level].w * sv.lv[level].h + blockDim.x - 1) / blockDim.x;
        if (b < n) break;
        b -= n;
    }
    if (level >= sv.levels) return;
    const int w = sv.lv[level].w, h = sv.lv[level].h;
    const int i = b * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const int x = i % w, y = i / w;
    const int set = sv.ts->idx;
    sv.nmap[set][level][i] = normal_at(sv.vmap[set][level], w, x, y, w, h);
}

}  // namespace

void launch_zrange(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st) {
    const int cells = (ex.w / 8) * (ex.h / 8);
    zr_init_kernel<<<dim3((cells + 255) / 256, nslots), 256, 0, st>>>(d_sv);
    const int gz = min(max((ex.max_pool + 255) / 256, 1), 304);
    zrange_kernel<<<dim3(gz, nslots), 256, 0, st>>>(d_sv);
}

void launch_march(const SessionView *d_sv, int nslots, const Extent &ex, float4 *vmap_ext, long long vmap_pitch,
                  const int *layouts, cudaStream_t st, uint8_t *rgb_ext, long long rgb_pitch) {
    const int tw = ray_tile_width(ex), th = kRayThreads / tw;
    // every slot's tiles fit: a smaller frame has fewer tiles per row and per column
    const dim3 g(((ex.w + tw - 1) / tw) * ((ex.h + th - 1) / th), nslots);
    if (rgb_ext) {
        if (layouts[GBF_VOXEL_REF])
            raycast_kernel<GBF_VOXEL_REF, true><<<g, kRayThreads, 0, st>>>(d_sv, vmap_ext, vmap_pitch, tw, rgb_ext,
                                                                           rgb_pitch);
        if (layouts[GBF_VOXEL_HALF])
            raycast_kernel<GBF_VOXEL_HALF, true><<<g, kRayThreads, 0, st>>>(d_sv, vmap_ext, vmap_pitch, tw, rgb_ext,
                                                                            rgb_pitch);
        if (layouts[GBF_VOXEL_SNORM])
            raycast_kernel<GBF_VOXEL_SNORM, true><<<g, kRayThreads, 0, st>>>(d_sv, vmap_ext, vmap_pitch, tw, rgb_ext,
                                                                             rgb_pitch);
        return;
    }
    if (layouts[GBF_VOXEL_REF])
        raycast_kernel<GBF_VOXEL_REF, false><<<g, kRayThreads, 0, st>>>(d_sv, vmap_ext, vmap_pitch, tw, nullptr, 0);
    if (layouts[GBF_VOXEL_HALF])
        raycast_kernel<GBF_VOXEL_HALF, false><<<g, kRayThreads, 0, st>>>(d_sv, vmap_ext, vmap_pitch, tw, nullptr, 0);
    if (layouts[GBF_VOXEL_SNORM])
        raycast_kernel<GBF_VOXEL_SNORM, false><<<g, kRayThreads, 0, st>>>(d_sv, vmap_ext, vmap_pitch, tw, nullptr, 0);
}

void launch_nmap_of(const float4 *vmap, long long vmap_pitch, float4 *nmap, long long nmap_pitch, int w, int h,
                    cudaStream_t st) {
    nmap_of_kernel<<<dim3((w + 127) / 128, h), 128, 0, st>>>(vmap, vmap_pitch, nmap, nmap_pitch, w, h);
}

int post_launches(const Extent &ex) { return ex.levels <= 3 ? 1 : ex.levels; }

void launch_post(const SessionView *d_sv, int nslots, const Extent &ex, cudaStream_t st) {
    if (ex.levels <= 3) {
        const int tiles = ((ex.w + kPostTile - 1) / kPostTile) * ((ex.h + kPostTile - 1) / kPostTile);
        post_pyramid_kernel<<<dim3(tiles, nslots), 256, 0, st>>>(d_sv);
        return;
    }
    int w = ex.w, h = ex.h, total = (w * h + 255) / 256;
    for (int l = 1; l < ex.levels; ++l) {
        w /= 2; h /= 2;
        vmap_down_kernel<<<dim3((w * h + 255) / 256, nslots), 256, 0, st>>>(d_sv, l);
        total += (w * h + 255) / 256;
    }
    nmap_all_kernel<<<dim3(total, nslots), 256, 0, st>>>(d_sv);
}

void launch_raycast(const SessionView *d_sv, int nslots, const Extent &ex, float4 *vmap_ext, long long vmap_pitch,
                    int post_pyramid, const int *layouts, cudaStream_t st, uint8_t *rgb_ext, long long rgb_pitch) {
    launch_zrange(d_sv, nslots, ex, st);
    launch_march(d_sv, nslots, ex, vmap_ext, vmap_pitch, layouts, st, rgb_ext, rgb_pitch);
    if (post_pyramid) launch_post(d_sv, nslots, ex, st);
}

}  // namespace gbf
