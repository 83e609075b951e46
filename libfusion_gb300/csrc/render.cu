// render.cu -- headless Phong shading of a vertex / normal map into RGBA8
// (renderPoint, renderSceneK, renderSceneTexturedK: src/tracking/cuda_imgproc.cu:17-108),
// the preview the reference draws through its GL viewer, written to a device buffer.
#include "gbf_device.cuh"
#include "gbf_kernels.h"

namespace gbf {

namespace {

// normalised(V) = V / V.norm() (include/math/vector_type.h:98-101, 198-201)
__device__ __forceinline__ float3 normalised(float3 v) {
    const float n = sqrtf((v.x * v.x + v.y * v.y) + v.z * v.z);
    return make_float3(v.x / n, v.y / n, v.z / n);
}

// renderPoint (cuda_imgproc.cu:17-48), float arithmetic as written.  In the
// reflection R = normalised(2 * normal * (normal * L) - L) the product
// `2 * normal` resolves to operator*(T, Vector3<U>) with T = int
// (vector_type.h:168-172), which returns Vector3<int>: 2 n truncated to
// integers.  That is reproduced.
__device__ __forceinline__ uchar4 render_point(float3 p, float3 n, float3 img) {
    float c0 = 4.f / 255.f, c1 = 2.f / 255.f, c2 = 2.f / 255.f;
    if (!isnan(p.x)) {
        const float Ka = 0.3f, Kd = 0.5f, Ks = 0.2f, sp = 20.f;
        const float Ax = img.x, Dx = img.y, Sx = img.z, Lx = 1.f;
        const float3 L = normalised(make_float3(5.f - p.x, 5.f - p.y, 5.f - p.z));  // light at (5, 5, 5)
        const float3 V = normalised(make_float3(0.f - p.x, 0.f - p.y, 0.f - p.z));
        const float nl = dot3(n, L);
        const int tx = (int)(n.x * 2.f), ty = (int)(n.y * 2.f), tz = (int)(n.z * 2.f);
        const float3 R = normalised(make_float3((float)tx * nl - L.x, (float)ty * nl - L.y, (float)tz * nl - L.z));
        const float rv = dot3(R, V);
        const float Ix =
            ((Ax * Ka) * Dx + ((Lx * Kd) * Dx) * fmaxf(0.f, nl)) + ((Lx * Ks) * Sx) * powf(fmaxf(0.f, rv), sp);
        c0 = c1 = c2 = Ix;
    }
    return make_uchar4((unsigned char)(__saturatef(c0) * 255.f), (unsigned char)(__saturatef(c1) * 255.f),
                       (unsigned char)(__saturatef(c2) * 255.f), 255);
}

__global__ void render_kernel(const float4 *vmap, long long vmap_pitch, const float4 *nmap, long long nmap_pitch,
                              const uint8_t *rgb, long long rgb_pitch, int rgb_stride, int w, int h, uchar4 *out,
                              long long out_pitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    const float4 v = reinterpret_cast<const float4 *>(reinterpret_cast<const char *>(vmap) + y * vmap_pitch)[x];
    const float4 n = reinterpret_cast<const float4 *>(reinterpret_cast<const char *>(nmap) + y * nmap_pitch)[x];
    float3 img = make_float3(1.f, 1.f, 1.f);
    if (rgb) {  // ToVector3f(image) / 255.f
        const uint8_t *c = rgb + y * rgb_pitch + (long long)x * rgb_stride;
        img = make_float3((float)c[0] / 255.f, (float)c[1] / 255.f, (float)c[2] / 255.f);
    }
    reinterpret_cast<uchar4 *>(reinterpret_cast<char *>(out) + y * out_pitch)[x] =
        render_point(make_float3(v.x, v.y, v.z), make_float3(n.x, n.y, n.z), img);
}

}  // namespace

void launch_render(const float4 *vmap, long long vmap_pitch, const float4 *nmap, long long nmap_pitch,
                   const uint8_t *rgb, long long rgb_pitch, int rgb_stride, int w, int h, uchar4 *out,
                   long long out_pitch, cudaStream_t st) {
    render_kernel<<<dim3((w + 127) / 128, h), 128, 0, st>>>(vmap, vmap_pitch, nmap, nmap_pitch, rgb, rgb_pitch,
                                                           rgb_stride, w, h, out, out_pitch);
}

}  // namespace gbf
