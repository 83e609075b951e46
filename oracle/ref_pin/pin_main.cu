// Pin program: runs the reference's own host-callable functions (compiled from
// the reference sources where they lie) on a fixed set of inputs and prints
// the results as JSON for tests/golden.  Built by oracle/ref_pin/build_ref.sh
// into oracle/_ref/; never part of the product.
#include <cstdio>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include "data_struct/map_struct.h"
#include "data_struct/intrinsic_matrix.h"
#include "voxel_hashing/device_tables.h"

using namespace fusion;

// Dump pin: a small chained map filled here, written by the reference's own
// MapStruct<false>::writeToDisk.  The blocks are laid out as a single-threaded
// createBlock would insert them in order (home bucket if free, else appended
// to the bucket's excess chain with offsets 1, 2, ...); the writer under test
// lays blocks out by the same rule, so its file must match byte for byte.
// The MapStruct constructors upload the map state to the device, so the host
// map is built in raw storage and only its host-side members are used.
static int dump_pin(const char *path) {
    const int nb = 16, ne = 24, nbk = 8;  // MapSize: blocks, hash entries, buckets
    const int pos[][3] = {{0, 0, 0},  {1, 0, 0},   {0, 1, 0},  {0, 0, 1},  {-1, -1, -1}, {5, -3, 2},
                          {-7, 4, 9}, {12, 12, 12}, {-20, 3, 0}, {100, -100, 50}, {3, 3, 3}, {-4, 8, -16}};
    const int n = sizeof(pos) / sizeof(pos[0]);
    alignas(MapStruct<false>) static unsigned char raw[sizeof(MapStruct<false>)];
    MapStruct<false> &m = *reinterpret_cast<MapStruct<false> *>(raw);
    std::memset(raw, 0, sizeof(raw));
    m.state.num_total_buckets_ = nbk;
    m.state.num_total_hash_entries_ = ne;
    m.state.num_total_voxel_blocks_ = nb;
    m.size.num_blocks = nb;
    m.size.num_hash_entries = ne;
    m.size.num_buckets = nbk;
    m.create();
    std::memset((void *)m.map.voxels_, 0, sizeof(Voxel) * nb * BLOCK_SIZE3);
    for (int i = 0; i < ne; ++i) {
        m.map.hash_table_[i].ptr_ = -1;
        m.map.hash_table_[i].offset_ = -1;
        m.map.hash_table_[i].pos_ = Vector3i(0, 0, 0);
    }
    for (int i = 0; i < nb; ++i) m.map.heap_mem_[i] = nb - i - 1;
    for (int i = 0; i < nbk; ++i) m.map.bucket_mutex_[i] = 0;
    int next_offset = 1;
    for (int b = 0; b < n; ++b) {
        Vector3i p(pos[b][0], pos[b][1], pos[b][2]);
        int cur = computeHash(p, nbk);
        HashEntry fresh(p, b * BLOCK_SIZE3, -1);
        if (m.map.hash_table_[cur].ptr_ == -1) {
            m.map.hash_table_[cur] = fresh;
        } else {
            while (m.map.hash_table_[cur].offset_ > 0) cur = nbk + m.map.hash_table_[cur].offset_ - 1;
            fresh.offset_ = 0;
            m.map.hash_table_[nbk + next_offset - 1] = fresh;
            m.map.hash_table_[cur].offset_ = next_offset++;
        }
        for (int i = 0; i < BLOCK_SIZE3; ++i) {
            Voxel &v = m.map.voxels_[b * BLOCK_SIZE3 + i];
            v.sdf = (short)(((b * 512 + i) * 37) % 65535 - 32767);
            v.weight = (float)((b * 7 + i) % 256);
            v.rgb = Vector3c((unsigned char)((b + i) % 256), (unsigned char)((b * 3 + i) % 256),
                             (unsigned char)((b * 5 + i) % 256));
        }
    }
    m.map.heap_mem_counter_[0] = nb - 1 - n;
    m.map.excess_counter_[0] = next_offset;
    m.writeToDisk(std::string(path));
    printf("{\"sizeof_voxel\": %d, \"sizeof_hash_entry\": %d, \"offsetof_voxel\": [%d, %d, %d], "
           "\"offsetof_hash_entry\": [%d, %d, %d], \"size\": [%d, %d, %d], \"blocks\": [",
           (int)sizeof(Voxel), (int)sizeof(HashEntry), (int)offsetof(Voxel, sdf), (int)offsetof(Voxel, weight),
           (int)offsetof(Voxel, rgb), (int)offsetof(HashEntry, ptr_), (int)offsetof(HashEntry, offset_),
           (int)offsetof(HashEntry, pos_), nb, ne, nbk);
    for (int b = 0; b < n; ++b) printf("%s[%d,%d,%d]", b ? "," : "", pos[b][0], pos[b][1], pos[b][2]);
    printf("]}\n");
    m.release();
    return 0;
}

int main(int argc, char **argv) {
    if (argc > 2 && std::strcmp(argv[1], "dump") == 0) return dump_pin(argv[2]);
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
