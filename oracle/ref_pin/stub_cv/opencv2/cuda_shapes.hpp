// Stand-ins for the few OpenCV 3.4 types the reference's mapping and tracking
// translation units name at their boundary, written from the shape of the
// public API (cv::cuda::PtrStep / PtrStepSz: a device pointer, a row step in
// bytes, and for PtrStepSz the columns and rows; cv::cuda::GpuMat: a pitched
// device image convertible to those views).  Only the device-side views have
// bodies: the reference kernels use them.  The host-side members are
// declared and never defined, because the pin program built with them is a
// device-only module (nvcc -cubin): the reference's own host functions are
// compiled for type checking and never called.
#pragma once
#include <cstddef>

typedef unsigned char uchar;

#define CV_8UC1 0
#define CV_32SC1 4
#define CV_32FC1 5
#define CV_32FC4 29
#define CV_8UC4 24

namespace cv {

struct Scalar {
    Scalar(double v0, double v1 = 0, double v2 = 0, double v3 = 0);
};

struct Size {
    int width, height;
    Size(int w, int h);
};

struct KeyPoint {
    float pt[2], size, angle, response;
    int octave, class_id;
};

class Mat {
public:
    template <typename T> T *ptr(int row = 0);
    template <typename T> const T *ptr(int row = 0) const;
};

enum { REDUCE_SUM = 0 };

namespace cuda {

template <typename T> struct DevPtr {
    T *data;
    __host__ __device__ DevPtr() : data(0) {}
    __host__ __device__ DevPtr(T *d) : data(d) {}
};

template <typename T> struct PtrStep : public DevPtr<T> {
    size_t step;
    __host__ __device__ PtrStep() : step(0) {}
    __host__ __device__ PtrStep(T *d, size_t s) : DevPtr<T>(d), step(s) {}
    __host__ __device__ T *ptr(int y = 0) { return (T *)((char *)DevPtr<T>::data + y * step); }
    __host__ __device__ const T *ptr(int y = 0) const {
        return (const T *)((const char *)DevPtr<T>::data + y * step);
    }
};

template <typename T> struct PtrStepSz : public PtrStep<T> {
    int cols, rows;
    __host__ __device__ PtrStepSz() : cols(0), rows(0) {}
    __host__ __device__ PtrStepSz(int r, int c, T *d, size_t s) : PtrStep<T>(d, s), cols(c), rows(r) {}
};

class GpuMat {
public:
    int flags, rows, cols;
    size_t step;
    uchar *data;
    bool empty() const;
    void create(int rows, int cols, int type);
    void create(Size size, int type);
    Size size() const;
    int type() const;
    GpuMat &setTo(Scalar s);
    void download(Mat &m) const;
    template <typename T> T *ptr(int y = 0);
    template <typename T> const T *ptr(int y = 0) const;
    template <typename T> operator PtrStepSz<T>() const;
    template <typename T> operator PtrStep<T>() const;
};

void reduce(const GpuMat &src, GpuMat &dst, int dim, int reduce_op, int dtype = -1);
void resize(const GpuMat &src, GpuMat &dst, Size dsize, double fx = 0, double fy = 0, int interpolation = 1);
void pyrDown(const GpuMat &src, GpuMat &dst);
void bilateralFilter(const GpuMat &src, GpuMat &dst, int kernel_size, float sigma_color, float sigma_spatial);

}  // namespace cuda
}  // namespace cv
