// Reference-kernel pin module: TSDF integration.  The reference's
// update_map_with_colour_kernel and update_map_weighted_kernel
// (src/voxel_hashing/depth_fusion.cu:288-428) are launched as they are, by
// name, with the launch shape of cuda::update / update_weighted (one 8x8 CTA
// per visible block, :488-500, :561-575).
#include "src/data_struct/map_struct.cu"
#include "src/voxel_hashing/depth_fusion.cu"
#include "pin_common.cuh"
