/*
 * oracle_common.c -- integer helpers and tables shared by both oracle
 * precisions.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 */
#include <limits.h>
#include <math.h>

#include "oracle.h"

/* computeHash (src/data_struct/map_struct.cu:143-148); the reference relies on
 * signed overflow wrapping, restated with unsigned 32-bit multiplies. */
int or_compute_hash(int x, int y, int z, int n) {
    unsigned ux = (unsigned)x * 73856093u, uy = (unsigned)y * 19349669u, uz = (unsigned)z * 83492791u;
    int res = (int)(ux ^ uy ^ uz);
    res %= n;
    return res < 0 ? res + n : res;
}

/* float -> int truncation with the saturation of the GPU conversion
 * (cvt.rzi.s32.f32: NaN -> 0, out of range -> INT_MIN / INT_MAX) */
int or_trunc_sat(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}

/* ToVector3i (include/math/vector_type.h:218-225) */
int or_floor_ref(float v) {
    int b = or_trunc_sat(v);
    return ((float)b > v) ? b - 1 : b;
}

/* voxelPosToBlockPos (map_struct.cu:626-636) */
void or_voxel_to_block(const int v[3], int out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = (v[i] < 0 ? v[i] - 7 : v[i]) / 8;
}

/* voxelPosToLocalPos (map_struct.cu:643-655) */
void or_voxel_to_local(const int v[3], int out[3]) {
    for (int i = 0; i < 3; ++i) {
        int r = v[i] % 8;
        out[i] = r < 0 ? r + 8 : r;
    }
}

/* localPosToLocalIdx (map_struct.cu:657-660) */
int or_local_idx(const int l[3]) { return l[2] * 64 + l[1] * 8 + l[0]; }

/* packFloat / unpackFloat (include/data_struct/voxel.h:36-44) */
short or_pack_sdf(float v) { return (short)or_trunc_sat(v * 32767.f); }
float or_unpack_sdf(short v) { return (float)v / 32767.f; }

/* Classic marching-cubes triangle table (public-domain Lorensen-Cline / Bourke
 * table, the same data as include/voxel_hashing/device_tables.h:25-280 of the
 * reference), packed: low nibble = triangle count, then one nibble per edge. */
static const unsigned long long k_tri[256] = {
#include "mc_table.inc"
};

/* cube corners (scene_mesh.cu:73-101) and edge endpoints (scene_mesh.cu:147-205) */
static const int k_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                  {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

/* edge_table derived from the corner signs: bit e set when edge e's corners differ */
int or_edge_table(int cube) {
    int m = 0;
    for (int e = 0; e < 12; ++e)
        if (((cube >> k_edge[e][0]) & 1) != ((cube >> k_edge[e][1]) & 1)) m |= 1 << e;
    return m;
}

int or_tri_table(int cube, int out[16]) {
    const unsigned long long p = k_tri[cube & 255];
    const int n = (int)(p & 0xF) * 3;
    for (int i = 0; i < 16; ++i) out[i] = -1;
    for (int i = 0; i < n; ++i) out[i] = (int)((p >> (4 + 4 * i)) & 0xF);
    return n;
}
