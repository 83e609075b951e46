// Stand-in for <sophus/se3.hpp> (Sophus, unpinned version) as the reference's
// mapping and tracking translation units use it: SE3d::cast<float>(),
// inverse() and matrix3x4() in their host functions, and the constructor of
// fusion::Matrix3x4 from a 3x4 Sophus::Matrix that matrix_type.h enables
// when SOPHUS_SE3_HPP is defined.  Host members are declared only (the pin
// program is a device-only module, where the reference's host functions are
// compiled for type checking and never called); the pin kernels pass their
// poses as plain float 3x4 matrices.
#ifndef SOPHUS_SE3_HPP
#define SOPHUS_SE3_HPP

namespace Sophus {

template <class T, int R, int C> struct Matrix {
    T m[R * C];
    __host__ __device__ T operator()(int r, int c) const { return m[r * C + c]; }
};

template <class T> class SE3 {
public:
    template <class U> SE3<U> cast() const;
    SE3 inverse() const;
    Matrix<T, 3, 4> matrix3x4() const;
};

typedef SE3<double> SE3d;
typedef SE3<float> SE3f;

}  // namespace Sophus

#endif
