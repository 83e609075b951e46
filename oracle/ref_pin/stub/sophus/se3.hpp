// Empty stand-in for <sophus/se3.hpp>.  The reference's include/math/
// vector_type.h includes it, but the host functions compiled for pinning
// (map_struct.cu converters and hash, voxel.h packing) use nothing from it;
// matrix_type.h guards its Sophus constructors with SOPHUS_SE3_HPP, left undefined.
#pragma once
