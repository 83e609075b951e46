// Reference-kernel pin module: marching cubes (src/voxel_hashing/
// scene_mesh.cu).  The functors are called as select_blocks_kernel,
// generate_vertex_and_normal_array_kernel, select_blocks_coloured_kernel and
// generate_vertex_and_colour_array_kernel call them (:250-258, :303-306,
// :590-598), with create_mesh_with_normal's / create_mesh_with_colour's
// launch shapes chosen by the caller (1024-thread CTAs over the hash table,
// then 8x8 CTAs on a (ceil(blocks / 16), 16) grid).
#include "src/data_struct/map_struct.cu"
#include "src/voxel_hashing/scene_mesh.cu"
#include "pin_common.cuh"

namespace pin {
template <class F>
__device__ inline F mesh_functor(fusion::Voxel *voxels, fusion::HashEntry *table, fusion::HashEntry *block_array,
                                 unsigned *block_count, unsigned *triangle_count, float *triangles) {
    F f;
    f.map_struct.heap_mem_ = nullptr;
    f.map_struct.excess_counter_ = nullptr;
    f.map_struct.heap_mem_counter_ = nullptr;
    f.map_struct.bucket_mutex_ = nullptr;
    f.map_struct.voxels_ = voxels;
    f.map_struct.hash_table_ = table;
    f.block_array = block_array;
    f.block_count = block_count;
    f.triangle_count = triangle_count;
    f.triangles = (fusion::Vector3f *)triangles;
    return f;
}
}  // namespace pin

extern "C" __global__ void pin_mesh_select(fusion::Voxel *voxels, fusion::HashEntry *table,
                                           fusion::HashEntry *block_array, unsigned *block_count) {
    auto f = pin::mesh_functor<fusion::cuda::BuildVertexArray>(voxels, table, block_array, block_count, nullptr,
                                                               nullptr);
    f.surface_normal = nullptr;
    f.select_blocks();
}

extern "C" __global__ void pin_mesh_normals(fusion::Voxel *voxels, fusion::HashEntry *table,
                                            fusion::HashEntry *block_array, unsigned *block_count,
                                            unsigned *triangle_count, float *triangles, float *normals) {
    auto f = pin::mesh_functor<fusion::cuda::BuildVertexArray>(voxels, table, block_array, block_count,
                                                               triangle_count, triangles);
    f.surface_normal = (fusion::Vector3f *)normals;
    f.template operator()<true>();
}

extern "C" __global__ void pin_mesh_colour_select(fusion::Voxel *voxels, fusion::HashEntry *table,
                                                  fusion::HashEntry *block_array, unsigned *block_count) {
    auto f = pin::mesh_functor<fusion::cuda::BuildVertexAndColourArray>(voxels, table, block_array, block_count,
                                                                        nullptr, nullptr);
    f.vertex_colour = nullptr;
    f.select_blocks();
}

extern "C" __global__ void pin_mesh_colour(fusion::Voxel *voxels, fusion::HashEntry *table,
                                           fusion::HashEntry *block_array, unsigned *block_count,
                                           unsigned *triangle_count, float *triangles, unsigned char *colours) {
    auto f = pin::mesh_functor<fusion::cuda::BuildVertexAndColourArray>(voxels, table, block_array, block_count,
                                                                        triangle_count, triangles);
    f.vertex_colour = (fusion::Vector3c *)colours;
    f();
}
