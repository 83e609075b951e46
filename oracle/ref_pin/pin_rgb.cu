// Reference-kernel pin module: the photometric row of every reference pixel,
// RgbReduction2::compute_jacobian (src/tracking/m_estimator.cu:313-391), one
// thread per pixel; out: 29 floats per pixel, the terms rgb_reduce_kernel2
// adds.  The fields are set as rgb_step sets them (:454-472).
#include "src/data_struct/map_struct.cu"
#include "src/tracking/m_estimator.cu"
#include "pin_common.cuh"

extern "C" __global__ void pin_rgb_rows(const float *curr_intensity, const float *last_intensity,
                                        const float *last_vmap, const float *curr_vmap, const float *dIdx,
                                        const float *dIdy, int cols, int rows, float stddev, const float *pose,
                                        float fx, float fy, float cx, float cy, float invfx, float invfy,
                                        float *out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cols * rows) return;
    fusion::RgbReduction2 rr;
    const size_t fstep = (size_t)cols * sizeof(float), vstep = (size_t)cols * 16;
    rr.cols = cols;
    rr.rows = rows;
    rr.N = cols * rows;
    rr.last_image = cv::cuda::PtrStep<float>((float *)last_intensity, fstep);
    rr.curr_image = cv::cuda::PtrStep<float>((float *)curr_intensity, fstep);
    rr.point_cloud = cv::cuda::PtrStep<fusion::Vector4f>((fusion::Vector4f *)curr_vmap, vstep);
    rr.last_vmap = cv::cuda::PtrStep<fusion::Vector4f>((fusion::Vector4f *)last_vmap, vstep);
    rr.dIdx = cv::cuda::PtrStep<float>((float *)dIdx, fstep);
    rr.dIdy = cv::cuda::PtrStep<float>((float *)dIdy, fstep);
    rr.pose = pin::m34(pose);
    rr.stddev = stddev;
    rr.fx = fx;
    rr.fy = fy;
    rr.cx = cx;
    rr.cy = cy;
    rr.invfx = invfx;
    rr.invfy = invfy;
    rr.compute_jacobian(k, out + (size_t)k * 29);
}
