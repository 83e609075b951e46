// Reference-kernel pin module: the ICP row of every reference pixel,
// ICPReduction::getRow (src/tracking/pose_estimator.cu:166-222), one thread
// per pixel; out: 29 floats per pixel (28 products of the row's upper
// triangle, then the correspondence flag), the terms icp_reduce_kernel adds.
// The fields are set as icp_reduce sets them (:282-297).
#include "src/data_struct/map_struct.cu"
#include "src/tracking/pose_estimator.cu"
#include "pin_common.cuh"

extern "C" __global__ void pin_icp_rows(const float *curr_vmap, const float *curr_nmap, const float *last_vmap,
                                        const float *last_nmap, int cols, int rows, const float *pose, float fx,
                                        float fy, float cx, float cy, float angle_thresh, float dist_thresh,
                                        float *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cols * rows) return;
    fusion::ICPReduction icp;
    const size_t step = (size_t)cols * 16;
    icp.curr_vmap_ = cv::cuda::PtrStep<fusion::Vector4f>((fusion::Vector4f *)curr_vmap, step);
    icp.curr_nmap_ = cv::cuda::PtrStep<fusion::Vector4f>((fusion::Vector4f *)curr_nmap, step);
    icp.last_vmap_ = cv::cuda::PtrStep<fusion::Vector4f>((fusion::Vector4f *)last_vmap, step);
    icp.last_nmap_ = cv::cuda::PtrStep<fusion::Vector4f>((fusion::Vector4f *)last_nmap, step);
    icp.cols = cols;
    icp.rows = rows;
    icp.N = cols * rows;
    icp.pose = pin::m34(pose);
    icp.angleThresh = angle_thresh;
    icp.distThresh = dist_thresh;
    icp.fx = fx;
    icp.fy = fy;
    icp.cx = cx;
    icp.cy = cy;
    icp.getRow(i, out + (size_t)i * 29);
}
