// ingest.cu -- frame ingest and tracking pyramids (DeviceImage::upload,
// src/tracking/device_image.cpp:146-181; kernels of src/tracking/cuda_imgproc.cu).
//
// Three launches per frame for all sessions of a batch:
//   1. ingest_l0:  u16 mm -> metres (System::process_images, src/system.cpp:43),
//                  rgb8 -> uchar4 + grey (device_image.cpp:161-162), bilateral
//                  filter of the tracking depth (cuda_imgproc.cu:197-200) from a
//                  shared-memory tile with a 2-pixel halo.
//   2. pyr_down:   per level, 2x2 mean of depth (cv::cuda::resize 0.5,
//                  cuda_imgproc.cu:202-205) and 5x5 binomial pyrDown of the
//                  intensity (cuda_imgproc.cu:207-210).  One launch per level.
//   3. level_maps: every level in one launch: dI/dx, dI/dy (computeDerivativeK,
//                  cuda_imgproc.cu:217-234), vertex map (backProjectDepthK,
//                  :249-263) and normal map (computeNMapK, :276-294), the normal
//                  computed from back-projected neighbours so no second pass.
// The OpenCV filters are third-party code absent here; they are restated from
// their documented definitions (bilateral: circular 5-tap window, Gaussian
// space/range weights; resize: pixel-centre bilinear at exactly 0.5; pyrDown:
// [1 4 6 4 1]/16 separable, reflect-101 border).
#include "gbf_device.cuh"
#include "gbf_kernels.h"

namespace gbf {

namespace {

constexpr int kTileW = 32, kTileH = 8, kHalo = 2;

__device__ __forceinline__ int reflect101(int i, int n) {
    if (i < 0) i = -i;
    if (i >= n) i = 2 * n - 2 - i;
    return i;
}

__device__ __forceinline__ int set_index(const SessionView &sv, int sel) {
    const int idx = sv.ts->idx;
    return sel ? idx : 1 - idx;
}

__global__ void __launch_bounds__(kTileW *kTileH) ingest_l0_kernel(const SessionView *__restrict__ svs, IngestArgs a) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    const int W = sv.lv[0].w, H = sv.lv[0].h;
    const int tiles_x = (W + kTileW - 1) / kTileW;
    const int tx0 = (blockIdx.x % tiles_x) * kTileW;
    const int ty0 = (blockIdx.x / tiles_x) * kTileH;
    if (ty0 >= H) return;  // uniform per CTA

    __shared__ float tile[kTileH + 2 * kHalo][kTileW + 2 * kHalo];
    const int nt = (kTileH + 2 * kHalo) * (kTileW + 2 * kHalo);
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        const int ly = i / (kTileW + 2 * kHalo), lx = i % (kTileW + 2 * kHalo);
        const int gx = reflect101(tx0 + lx - kHalo, W), gy = reflect101(ty0 + ly - kHalo, H);
        float z;
        if (a.src == 0) {
            z = (float)sv.in_depth[(size_t)gy * W + gx] * 0.001f;
        } else if (a.src == 1) {
            const uint16_t *row = reinterpret_cast<const uint16_t *>(static_cast<const char *>(a.depth) + gy * a.depth_pitch);
            z = (float)row[gx] * 0.001f;
        } else {
            const float *row = reinterpret_cast<const float *>(static_cast<const char *>(a.depth) + gy * a.depth_pitch);
            z = row[gx];
        }
        tile[ly][lx] = z;
    }
    __syncthreads();

    const int lx = threadIdx.x % kTileW, ly = threadIdx.x / kTileW;
    const int x = tx0 + lx, y = ty0 + ly;
    if (x >= W || y >= H) return;
    const size_t p = (size_t)y * W + x;
    const float c = tile[ly + kHalo][lx + kHalo];
    sv.depth_raw[p] = c;

    float filt = c;
    if (sv.bilateral) {
        // circular window of radius 2 (cv::cuda::bilateralFilter(src, dst, 5, 1, 1))
        const float ks = -0.5f, kc = -0.5f;  // -1/(2 sigma^2), sigma_space = sigma_colour = 1
        float s1 = 0.f, s2 = 0.f;
#pragma unroll
        for (int dy = -2; dy <= 2; ++dy) {
#pragma unroll
            for (int dx = -2; dx <= 2; ++dx) {
                const int sp = dx * dx + dy * dy;
                if (sp > 4) continue;
                const float v = tile[ly + kHalo + dy][lx + kHalo + dx];
                const float d = v - c;
                const float w = expf((float)sp * ks + (d * d) * kc);
                s1 += w * v;
                s2 += w;
            }
        }
        filt = s1 / s2;
    }
    sv.depth[0][p] = filt;

    uint8_t r, g, b;
    if (a.src == 0) {
        const uint8_t *px = sv.in_rgb + p * 3;
        r = px[0]; g = px[1]; b = px[2];
    } else {
        const uint8_t *px = a.rgb + y * a.rgb_pitch + (size_t)x * 3;
        r = px[0]; g = px[1]; b = px[2];
    }
    sv.rgb4[p] = make_uchar4(r, g, b, 0);
    // cv::COLOR_RGB2GRAY on CV_32FC3: 0.299 R + 0.587 G + 0.114 B
    const float grey = (0.299f * (float)r + 0.587f * (float)g) + 0.114f * (float)b;
    sv.inten[set_index(sv, a.set_sel)][0][p] = grey;
}

__global__ void pyr_down_kernel(const SessionView *__restrict__ svs, int set_sel, int level) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active || level >= sv.levels) return;
    const int w = sv.lv[level].w, h = sv.lv[level].h;
    const int pw = sv.lv[level - 1].w, ph = sv.lv[level - 1].h;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const int x = i % w, y = i / w;
    const int set = set_index(sv, set_sel);

    // depth: 2x2 mean (resize by 0.5, pixel-centre bilinear)
    const float *sd = sv.depth[level - 1];
    const float a0 = sd[(size_t)(2 * y) * pw + 2 * x], a1 = sd[(size_t)(2 * y) * pw + 2 * x + 1];
    const float a2 = sd[(size_t)(2 * y + 1) * pw + 2 * x], a3 = sd[(size_t)(2 * y + 1) * pw + 2 * x + 1];
    sv.depth[level][i] = (((a0 + a1) + a2) + a3) * 0.25f;

    // intensity: 5x5 binomial, reflect-101, sample at (2x, 2y)
    const float *si = sv.inten[set][level - 1];
    int xs[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xs[k] = reflect101(2 * x + k - 2, pw);
    float hrow[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const float *row = si + (size_t)reflect101(2 * y + j - 2, ph) * pw;
        hrow[j] = (((row[xs[0]] + 4.f * row[xs[1]]) + 6.f * row[xs[2]]) + 4.f * row[xs[3]]) + row[xs[4]];
    }
    sv.inten[set][level][i] = ((((hrow[0] + 4.f * hrow[1]) + 6.f * hrow[2]) + 4.f * hrow[3]) + hrow[4]) * (1.f / 256.f);
}

// backProjectDepthK (cuda_imgproc.cu:249-263)
__device__ __forceinline__ float4 back_project(const float *depth, int w, int x, int y, const LevelK &K) {
    const float z = depth[(size_t)y * w + x];
    if (z > 0.3f && z < 5.0f)
        return make_float4((z * ((float)x - K.cx)) * K.invfx, (z * ((float)y - K.cy)) * K.invfy, z, 1.0f);
    return make_float4(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff), __int_as_float(0x7fffffff), -1.0f);
}

__device__ __forceinline__ float4 normal_from(float4 v00, float4 v01, float4 v10, float4 v11) {
    const float3 a = make_float3(v01.x - v00.x, v01.y - v00.y, v01.z - v00.z);
    const float3 b = make_float3(v11.x - v10.x, v11.y - v10.y, v11.z - v10.z);
    const float3 n = cross3(a, b);
    const float l = norm3(n.x, n.y, n.z);
    return make_float4(n.x / l, n.y / l, n.z / l, 1.f);
}

// Integration test and weight of the frame's pixel for the normal-weighted
// update (update_map_weighted_kernel, depth_fusion.cu:390-405): raw depth,
// level-0 normal of the filtered depth; rejected pixels carry NaN depth.
__device__ __forceinline__ void fuse_weight(const SessionView &sv, int i, float4 n) {
    const float dist = sv.depth_raw[i];
    const bool ok = !(isnan(dist) || isnan(n.x) || dist > sv.zmax_u || dist < sv.zmin_u);
    const float w = fabsf(sinf(n.z)) / (dist * dist);
    sv.fuse_px[i] = make_float2(ok ? dist : __int_as_float(0x7fffffff), w);
}

__global__ void __launch_bounds__(256, 8) level_maps_kernel(const SessionView *__restrict__ svs, int set_sel, int tiles_per_level0) {
    const SessionView &sv = svs[blockIdx.y];
    if (!sv.active) return;
    // flatten the levels: level l owns ceil(P_l / blockDim) CTAs
    int b = blockIdx.x, level = 0;
    for (; level < sv.levels; ++level) {
        const int n = (sv.lv[level].w * sv.lv[level].h + blockDim.x - 1) / blockDim.x;
        if (b < n) break;
        b -= n;
    }
    if (level >= sv.levels) return;
    const LevelK K = sv.lv[level];
    const int i = b * blockDim.x + threadIdx.x;
    if (i >= K.w * K.h) return;
    const int x = i % K.w, y = i / K.w;
    const int set = set_index(sv, set_sel);
    const float *I = sv.inten[set][level];
    const float *D = sv.depth[level];

    const float nanf_ = __int_as_float(0x7fffffff);
    if (x < K.w - 1 && y < K.h - 1) {
        const int x10 = max(x - 1, 0), y10 = max(y - 1, 0);
        const float gx = (I[(size_t)y * K.w + x + 1] - I[(size_t)y * K.w + x10]) * 0.5f;
        const float gy = (I[(size_t)(y + 1) * K.w + x] - I[(size_t)y10 * K.w + x]) * 0.5f;
        sv.gx[level][i] = gx;
        sv.gy[level][i] = gy;
        sv.igd[set][level][i] = make_float4(I[i], gx, gy, 0.f);
        const float4 v00 = back_project(D, K.w, x10, y, K);
        const float4 v01 = back_project(D, K.w, x + 1, y, K);
        const float4 v10 = back_project(D, K.w, x, y10, K);
        const float4 v11 = back_project(D, K.w, x, y + 1, K);
        const float4 n = normal_from(v00, v01, v10, v11);
        sv.nmap[set][level][i] = n;
        if (level == 0 && set_sel == 0) fuse_weight(sv, i, n);
    } else {
        // the reference leaves the last row / column unwritten; write invalid
        sv.gx[level][i] = 0.f;
        sv.gy[level][i] = 0.f;
        sv.igd[set][level][i] = make_float4(I[i], 0.f, 0.f, 0.f);
        sv.nmap[set][level][i] = make_float4(nanf_, nanf_, nanf_, nanf_);
        if (level == 0 && set_sel == 0) fuse_weight(sv, i, make_float4(nanf_, nanf_, nanf_, nanf_));
    }
    sv.vmap[set][level][i] = back_project(D, K.w, x, y, K);
}

}  // namespace

void launch_ingest(const SessionView *d_sv, int nslots, const Extent &ex, const IngestArgs &a, cudaStream_t st) {
    const int tiles = ((ex.w + kTileW - 1) / kTileW) * ((ex.h + kTileH - 1) / kTileH);
    ingest_l0_kernel<<<dim3(tiles, nslots), kTileW * kTileH, 0, st>>>(d_sv, a);
    int w = ex.w, h = ex.h;
    for (int l = 1; l < ex.levels; ++l) {
        w /= 2; h /= 2;
        pyr_down_kernel<<<dim3((w * h + 255) / 256, nslots), 256, 0, st>>>(d_sv, a.set_sel, l);
    }
    int total = 0;
    w = ex.w; h = ex.h;
    for (int l = 0; l < ex.levels; ++l) {
        total += (w * h + 255) / 256;
        w /= 2; h /= 2;
    }
    level_maps_kernel<<<dim3(total, nslots), 256, 0, st>>>(d_sv, a.set_sel, 0);
}

}  // namespace gbf
