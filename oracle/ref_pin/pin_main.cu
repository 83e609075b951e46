// Pin driver: runs the reference's own host-callable functions (compiled from
// the reference sources where they lie) on a fixed set of inputs and prints
// the results as JSON for tests/golden.  Built by oracle/ref_pin/build_ref.sh
// into oracle/_ref/; never part of the product.
#include <cstdio>
#include <cmath>
#include "data_struct/map_struct.h"
#include "data_struct/intrinsic_matrix.h"
#include "voxel_hashing/device_tables.h"

using namespace fusion;

int main() {
    const int coords[] = {0, 1, -1, 7, -7, 8, -8, 9, -9, 100, -100, 4097, -4097, 65535, -65536, 1048575, -1048575,
                          2147483647, -2147483647 - 1, 123456789, -987654321};
    const int nc = sizeof(coords) / sizeof(coords[0]);
    const int buckets[] = {1, 7, 200000, 262144, 2097152, 2147483647};
    printf("{\n  \"hash\": [");
    bool first = true;
    for (int b : buckets)
        for (int i = 0; i < nc; ++i)
            for (int j = 0; j < nc; j += 3)
                for (int k = 0; k < nc; k += 5) {
                    Vector3i p(coords[i], coords[j], coords[k]);
                    printf("%s[%d,%d,%d,%d,%d]", first ? "" : ",", coords[i], coords[j], coords[k], b,
                           computeHash(p, b));
                    first = false;
                }
    printf("],\n  \"voxel_block_local\": [");
    first = true;
    for (int i = 0; i < nc; ++i) {
        if (coords[i] < -2147483640 ) continue;  // voxelPosToBlockPos subtracts 7
        Vector3i v(coords[i], coords[(i + 3) % nc], coords[(i + 7) % nc]);
        if (v.y < -2147483640 || v.z < -2147483640) continue;
        Vector3i bp = voxelPosToBlockPos(v), lp = voxelPosToLocalPos(v);
        printf("%s[%d,%d,%d,%d,%d,%d,%d,%d,%d,%d]", first ? "" : ",", v.x, v.y, v.z, bp.x, bp.y, bp.z, lp.x, lp.y,
               lp.z, localPosToLocalIdx(lp));
        first = false;
    }
    printf("],\n  \"world_to_voxel\": [");
    const float pts[] = {0.f, 0.005f, -0.005f, 0.01f, -0.01f, 0.0149999f, 1.234567f, -1.234567f, 3.99999f, -0.0000001f,
                         2.5f, -2.5f, 0.07999999f, 0.08f};
    const float vs[] = {0.004f, 0.005f, 0.008f, 0.01f, 0.016f};
    first = true;
    for (float v : vs)
        for (float x : pts) {
            Vector3i r = worldPtToVoxelPos(Vector3f(x, -x, x * 0.5f), v);
            printf("%s[%.9g,%.9g,%d,%d,%d]", first ? "" : ",", x, v, r.x, r.y, r.z);
            first = false;
        }
    printf("],\n  \"pack_sdf\": [");
    const float sd[] = {0.f, 1.f, -1.f, 0.5f, -0.5f, 0.33333334f, -0.33333334f, 1e-5f, -1e-5f, 0.99999994f, 3.0517578e-05f};
    first = true;
    for (float s : sd) {
        Voxel vx;
        vx.setSDF(s);
        vx.setWeight(300.f);
        printf("%s[%.9g,%d,%.9g,%.9g]", first ? "" : ",", s, (int)vx.sdf, vx.getSDF(), vx.getWeight());
        first = false;
    }
    printf("],\n  \"intrinsics_pyr\": [");
    IntrinsicMatrix K(640, 480, 525.f, 525.f, 319.5f, 239.5f);
    for (int l = 0; l < 5; ++l) {
        printf("%s[%d,%d,%.9g,%.9g,%.9g,%.9g,%.9g,%.9g]", l ? "," : "", K.width, K.height, K.fx, K.fy, K.cx, K.cy,
               K.invfx, K.invfy);
        K = K.pyr_down();
    }
    printf("],\n  \"edge_table\": [");
    for (int i = 0; i < 256; ++i) printf("%s%d", i ? "," : "", edge_table[i]);
    printf("],\n  \"triangle_table\": [");
    for (int i = 0; i < 256; ++i) {
        printf("%s[", i ? "," : "");
        for (int j = 0; j < 16; ++j) printf("%s%d", j ? "," : "", triangle_table[i][j]);
        printf("]");
    }
    printf("]\n}\n");
    return 0;
}
