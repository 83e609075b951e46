// mesh.cu -- marching cubes over all allocated blocks (src/voxel_hashing/
// scene_mesh.cu:14-643, tables include/voxel_hashing/device_tables.h).
//
// GB300 design: two passes over the allocated-block list (ids 0..n-1 of the
// pool; the reference instead compacts the whole hash table, scene_mesh.cu:24-52).
//   count  one CTA (512 threads, one per voxel) per block stages the block and
//          its +x/+y/+z halo (9x9x9 sdf + validity) in shared memory with 7
//          neighbour lookups, classifies every voxel's cube and sums the
//          block's triangles.
//   scan   exclusive prefix of the per-block counts (one CTA).
//   emit   restages, takes the in-block prefix of the voxels' triangle counts
//          and writes every triangle at a fixed position.
// Output order is deterministic (block id, voxel index, table order); the
// reference appends with one global atomicAdd per triangle (scene_mesh.cu:231).
// Vertex arithmetic follows make_vertex (scene_mesh.cu:119-209) exactly.
#include "gbf_device.cuh"
#include "gbf_kernels.h"

namespace gbf {

namespace {

// Triangle table of classic marching cubes (the public-domain Lorensen-Cline /
// Bourke table, identical to the reference's triangle_table so that the mesh
// topology matches bit for bit).  Packed: low nibble = number of triangles,
// then one nibble per edge index, three per triangle, in table order.
__constant__ unsigned long long kTriPacked[256] = {
    0x0000000000000000ull, 0x0000000000003801ull, 0x0000000000009101ull, 0x0000000001893812ull,
    0x000000000000a211ull, 0x000000000a213802ull, 0x000000000920a292ull, 0x00000089a8a23823ull,
    0x0000000000002b31ull, 0x0000000000b82b02ull, 0x000000000b320912ull, 0x000000b89b912b13ull,
    0x0000000003ab1a32ull, 0x000000ab8a801a03ull, 0x0000009ab9b30933ull, 0x000000000b8aa892ull,
    0x0000000000008741ull, 0x0000000004370342ull, 0x0000000007489102ull, 0x0000001371749143ull,
    0x000000000748a212ull, 0x000000a214037433ull, 0x000000748209a293ull, 0x0004973727929a24ull,
    0x0000000002b37482ull, 0x00000040242b74b3ull, 0x000000b327481093ull, 0x0001292b9b49b744ull,
    0x000000487ab31a33ull, 0x0004b7401b41ab14ull, 0x00030bab9b098744ull, 0x000000ab99b4b743ull,
    0x0000000000004591ull, 0x0000000003804592ull, 0x0000000000514502ull, 0x0000005135384583ull,
    0x000000000459a212ull, 0x000000594a218033ull, 0x000000204245a253ull, 0x0008434535235a24ull,
    0x000000000b324592ull, 0x000000594b802b03ull, 0x000000b325104503ull, 0x000584b828525124ull,
    0x00000045931ab3a3ull, 0x000ab81a81805944ull, 0x00030bab5b050454ull, 0x000000b8aa858453ull,
    0x0000000009758792ull, 0x0000003753590393ull, 0x0000007517108703ull, 0x0000000007533512ull,
    0x00000021a7598793ull, 0x00037503505921a4ull, 0x00025a7585282084ull, 0x0000007533525a23ull,
    0x0000002b39875973ull, 0x000b720292797594ull, 0x000751871810b324ull, 0x00000051771b12b3ull,
    0x000b3a31a7588594ull, 0x0aba010b79050755ull, 0x07570805a30b0ab5ull, 0x0000000005b75ab2ull,
    0x00000000000056a1ull, 0x0000000006a53802ull, 0x0000000006a51092ull, 0x0000006a58913813ull,
    0x0000000001625612ull, 0x0000008036215613ull, 0x0000006206095693ull, 0x0008236252858954ull,
    0x00000000056ab322ull, 0x00000056a02b80b3ull, 0x0000006a5b329103ull, 0x000b892b92916a54ull,
    0x000000315356b363ull, 0x0006b51505b0b804ull, 0x0009505606306b34ull, 0x00000089bb969563ull,
    0x0000000008746a52ull, 0x000000a563740343ull, 0x0000007486a50913ull, 0x00049737179156a4ull,
    0x0000008741562163ull, 0x0007434036255214ull, 0x0006205605097484ull, 0x9626959234979375ull,
    0x00000056a4872b33ull, 0x000b720242746a54ull, 0x0006a5b328749104ull, 0x6a54b7b492b91295ull,
    0x0006b51535b37484ull, 0xb404b7b016b5b155ull, 0x74836b6305609505ull, 0x0009b7974b969564ull,
    0x000000000a4694a2ull, 0x000000380a946a43ull, 0x00000004606a10a3ull, 0x000a164686181384ull,
    0x0000004624219413ull, 0x0004629429218034ull, 0x0000000006244202ull, 0x0000006244282383ull,
    0x00000032b46a94a3ull, 0x0006a4a94b822804ull, 0x000a164606102b34ull, 0x1b8b12184a161465ull,
    0x00036b3196394694ull, 0x14641916b0181b85ull, 0x0000004600636b33ull, 0x00000000086b8462ull,
    0x000000a98a876a73ull, 0x000a76a907a03704ull, 0x0000818717a176a4ull, 0x00000037117a76a3ull,
    0x0007689818616214ull, 0x9373909761929625ull, 0x0000002066070873ull, 0x0000000002762372ull,
    0x00076898a86ab324ull, 0x7a9a76790b727025ull, 0xb32a767a18710815ull, 0x00017616a71b12b4ull,
    0x63136b6197686985ull, 0x00000000076b1902ull, 0x00006b0b36070874ull, 0x0000000000006b71ull,
    0x000000000000b671ull, 0x00000000067b8032ull, 0x00000000067b9102ull, 0x00000067b1389183ull,
    0x0000000007b621a2ull, 0x0000007b6803a213ull, 0x0000007b69a20923ull, 0x00089a38a3a27b64ull,
    0x0000000007263272ull, 0x0000000260678073ull, 0x0000009107326723ull, 0x0006788916812614ull,
    0x00000073171a67a3ull, 0x000801781a7167a4ull, 0x0007a69a0a707304ull, 0x0000009a88a7a673ull,
    0x00000000068b4862ull, 0x000000640603b633ull, 0x000000109648b683ull, 0x00063b1393696494ull,
    0x0000001a28b64863ull, 0x000640b60b03a214ull, 0x0009a2920b648b44ull, 0x36463b34923a39a5ull,
    0x0000002642483283ull, 0x0000000002642402ull, 0x0008346424320914ull, 0x0000006422414913ull,
    0x0001a66481683184ull, 0x00000040660a01a3ull, 0x39a9303a68343645ull, 0x0000000004a649a2ull,
    0x000000000b675942ull, 0x00000067b5943803ull, 0x000000b670451053ull, 0x00051345343867b4ull,
    0x000000b6721a4593ull, 0x000594380a217b64ull, 0x000204a24a45b674ull, 0x67b25a5234538435ull,
    0x0000009452673273ull, 0x0007862606804594ull, 0x0000450516732634ull, 0x8515848127868265ull,
    0x00073167161a4594ull, 0x459078701671a615ull, 0xa737a6a305a4a045ull, 0x000a84a458a7a674ull,
    0x00000098b9b65963ull, 0x000590650360b634ull, 0x000b65510b508b04ull, 0x0000001355363b63ull,
    0x00065b8b9b59a214ull, 0xa21965690b603b05ull, 0x52025a50865b58b5ull, 0x00035a3a25363b64ull,
    0x0002832658259854ull, 0x0000002600696593ull, 0x8262838650818515ull, 0x0000000006126512ull,
    0x698965683a616315ull, 0x00006505960a01a4ull, 0x000000000a658302ull, 0x00000000000065a1ull,
    0x000000000b57a5b2ull, 0x00000003857ba5b3ull, 0x000000091ba57b53ull, 0x0001381897ba57a4ull,
    0x00000015717b21b3ull, 0x000b275717213804ull, 0x0007b22097295794ull, 0x289823295b272575ull,
    0x000000573532a523ull, 0x00052a5782580284ull, 0x0002a37353a51094ull, 0x25752a2781292895ull,
    0x0000000005735312ull, 0x0000005711707803ull, 0x0000007355393093ull, 0x0000000007957892ull,
    0x0000008ba8a54853ull, 0x00003bba50b54054ull, 0x00054aba8a489104ull, 0x41314943b54a4ba5ull,
    0x0008548b25821524ull, 0xb151b2b543b0b405ull, 0x58b8545b29505205ull, 0x0000000003b25492ull,
    0x000483543253a524ull, 0x0000000244252a53ull, 0x910854583a532a35ull, 0x0002492914252a54ull,
    0x0000001533585483ull, 0x0000000005015402ull, 0x0005305093585484ull, 0x0000000000005491ull,
    0x000000ba9b947b43ull, 0x000ba97b97943804ull, 0x000b470414b1ba14ull, 0x4bab474a18434135ull,
    0x000219b294b97b44ull, 0x3801b2b197b94795ull, 0x00000004224b47b3ull, 0x00042343824b47b4ull,
    0x000947732972a924ull, 0x70207872a4797a95ull, 0xa040a1a472a3a735ull, 0x0000000004782a12ull,
    0x0000003177141943ull, 0x0001781807141944ull, 0x0000000003473042ull, 0x0000000000007841ull,
    0x0000000008ba8a92ull, 0x000000a9bb939033ull, 0x000000ba88a0a103ull, 0x000000000a3ba132ull,
    0x0000008b99b1b213ull, 0x0009b2921b939034ull, 0x000000000b08b202ull, 0x000000000000b231ull,
    0x00000098aa828323ull, 0x0000000002902a92ull, 0x0008a1810a828324ull, 0x0000000000002a11ull,
    0x0000000008198312ull, 0x0000000000001901ull, 0x0000000000008301ull, 0x0000000000000000ull,
};

// Cube corners in make_vertex order (scene_mesh.cu:73-101) and the corner
// pair of each of the 12 edges (scene_mesh.cu:147-205).
__constant__ int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                 {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

constexpr int kHaloSide = 9;
constexpr int kHaloCells = kHaloSide * kHaloSide * kHaloSide;

struct MeshSmem {
    float sdf[kHaloCells];
    unsigned char ok[kHaloCells];
    unsigned char rgb[kHaloCells][3];
    int nb[8];
    int tri[kBlockVoxels];
    int warp_tot[kBlockVoxels / 32];
};

__device__ __forceinline__ int edge_mask(int ci) {
    int m = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        const int a = (ci >> kEdge[e][0]) & 1, b = (ci >> kEdge[e][1]) & 1;
        if (a != b) m |= 1 << e;
    }
    return m;
}

// Stage block `id` plus its +x/+y/+z halo; validity per the mesh mode:
// weight != 0 (scene_mesh.cu:58) or weight > 1e-3 for colour (scene_mesh.cu:397).
template <int LAYOUT>
__device__ void stage_block(const SessionView &sv, int id, int mode, MeshSmem &sm) {
    const int4 bc = sv.bcoord[id];
    if (threadIdx.x < 8) {
        const int dx = threadIdx.x & 1, dy = (threadIdx.x >> 1) & 1, dz = (threadIdx.x >> 2) & 1;
        sm.nb[threadIdx.x] = (threadIdx.x == 0) ? id : find_block(sv, bc.x + dx, bc.y + dy, bc.z + dz);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < kHaloCells; c += blockDim.x) {
        const int x = c % kHaloSide, y = (c / kHaloSide) % kHaloSide, z = c / (kHaloSide * kHaloSide);
        const int nbi = (x >> 3) | ((y >> 3) << 1) | ((z >> 3) << 2);
        const int nid = sm.nb[nbi];
        bool ok = false;
        float s = 0.f;
        uchar4 col = make_uchar4(0, 0, 0, 0);
        if (nid >= 0) {
            const size_t vi = (size_t)nid * kBlockVoxels + (z & 7) * 64 + (y & 7) * 8 + (x & 7);
            float w;
            s = load_sdf<LAYOUT>(sv, vi, w);
            ok = (mode == GBF_MESH_COLOUR) ? ((double)w > 1e-3) : (w != 0.f);
            if (mode == GBF_MESH_COLOUR) col = sv.vox_rgb[vi];
        }
        sm.sdf[c] = s;
        sm.ok[c] = ok;
        sm.rgb[c][0] = col.x; sm.rgb[c][1] = col.y; sm.rgb[c][2] = col.z;
    }
    __syncthreads();
}

__device__ __forceinline__ int cube_of(const MeshSmem &sm, int li, float s[8], int corner_cell[8]) {
    const int x = li & 7, y = (li >> 3) & 7, z = li >> 6;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int c = (x + kCorner[k][0]) + (y + kCorner[k][1]) * kHaloSide + (z + kCorner[k][2]) * kHaloSide * kHaloSide;
        corner_cell[k] = c;
        if (!sm.ok[c]) return -1;
        s[k] = sm.sdf[c];
    }
    int ci = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (s[k] < 0) ci |= 1 << k;
    return ci;
}

template <int LAYOUT>
__global__ void __launch_bounds__(kBlockVoxels) mesh_count_kernel(const SessionView *__restrict__ svs, int mode, int *counts) {
    const SessionView &sv = svs[0];
    const int n = min(sv.ctr[C_NUSED], sv.pool);
    __shared__ MeshSmem sm;
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        stage_block<LAYOUT>(sv, b, mode, sm);
        float s[8];
        int cc[8];
        const int ci = cube_of(sm, threadIdx.x, s, cc);
        int t = 0;
        if (ci > 0 && edge_mask(ci) != 0) t = (int)(kTriPacked[ci] & 0xF);
        // block sum
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
        if ((threadIdx.x & 31) == 0) sm.warp_tot[threadIdx.x >> 5] = t;
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int w = 0; w < kBlockVoxels / 32; ++w) tot += sm.warp_tot[w];
            counts[b] = tot;
        }
        __syncthreads();
    }
}

// exclusive scan of counts[0..n) in place, total into C_MESH_TRIS (one CTA)
__global__ void mesh_scan_kernel(const SessionView *__restrict__ svs, int *counts) {
    const SessionView &sv = svs[0];
    const int n = min(sv.ctr[C_NUSED], sv.pool);
    __shared__ long long carry;
    __shared__ int wsum[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = (i < n) ? counts[i] : 0;
        // inclusive warp scan
        int x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if ((threadIdx.x & 31) >= off) x += y;
        }
        if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int w = (threadIdx.x < (int)(blockDim.x >> 5)) ? wsum[threadIdx.x] : 0;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, off);
                if (threadIdx.x >= off) w += y;
            }
            wsum[threadIdx.x] = w;
        }
        __syncthreads();
        const int wid = threadIdx.x >> 5;
        const long long excl = carry + (wid ? wsum[wid - 1] : 0) + (x - v);
        if (i < n) counts[i] = (int)excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        counts[n] = (int)carry;
        sv.ctr[C_MESH_TRIS] = (int)carry;
    }
}

template <int LAYOUT>
__global__ void __launch_bounds__(kBlockVoxels) mesh_emit_kernel(const SessionView *__restrict__ svs, int mode, const int *offsets,
                                                                 float3 *vtx, void *attr, long long max_tris) {
    const SessionView &sv = svs[0];
    const int n = min(sv.ctr[C_NUSED], sv.pool);
    __shared__ MeshSmem sm;
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        if (offsets[b] >= max_tris || offsets[b + 1] == offsets[b]) continue;  // uniform per CTA
        stage_block<LAYOUT>(sv, b, mode, sm);
        float s[8];
        int cc[8];
        const int li = threadIdx.x;
        const int ci = cube_of(sm, li, s, cc);
        const int em = (ci > 0) ? edge_mask(ci) : 0;
        const unsigned long long packed = (em != 0) ? kTriPacked[ci] : 0ull;
        const int t = (int)(packed & 0xF);
        // in-block exclusive prefix of t (voxel order)
        int x = t;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if ((li & 31) >= off) x += y;
        }
        if ((li & 31) == 31) sm.warp_tot[li >> 5] = x;
        __syncthreads();
        if (li < 32) {
            int w = (li < kBlockVoxels / 32) ? sm.warp_tot[li] : 0;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, off);
                if (li >= off) w += y;
            }
            if (li < kBlockVoxels / 32) sm.warp_tot[li] = w;
        }
        __syncthreads();
        const long long first = (long long)offsets[b] + ((li >> 5) ? sm.warp_tot[(li >> 5) - 1] : 0) + (x - t);
        if (t > 0) {
            const int4 bc = sv.bcoord[b];
            const int px = bc.x * 8 + (li & 7), py = bc.y * 8 + ((li >> 3) & 7), pz = bc.z * 8 + (li >> 6);
            const float fx = (float)px, fy = (float)py, fz = (float)pz;
            // interpolate_sdf (scene_mesh.cu:108-117)
            float3 ev[12];
#pragma unroll
            for (int e = 0; e < 12; ++e) {
                if (!((em >> e) & 1)) continue;
                const float v1 = s[kEdge[e][0]], v2 = s[kEdge[e][1]];
                float val;
                if ((double)fabsf(0 - v1) < 1e-6) val = 0;
                else if ((double)fabsf(0 - v2) < 1e-6) val = 1;
                else if ((double)fabsf(v1 - v2) < 1e-6) val = 0;
                else val = (0 - v1) / (v2 - v1);
                float ox, oy, oz;
                switch (e) {
                    case 0: ox = val; oy = 0; oz = 0; break;
                    case 1: ox = 1; oy = val; oz = 0; break;
                    case 2: ox = 1 - val; oy = 1; oz = 0; break;
                    case 3: ox = 0; oy = 1 - val; oz = 0; break;
                    case 4: ox = val; oy = 0; oz = 1; break;
                    case 5: ox = 1; oy = val; oz = 1; break;
                    case 6: ox = 1 - val; oy = 1; oz = 1; break;
                    case 7: ox = 0; oy = 1 - val; oz = 1; break;
                    case 8: ox = 0; oy = 0; oz = val; break;
                    case 9: ox = 1; oy = 0; oz = val; break;
                    case 10: ox = 1; oy = 1; oz = val; break;
                    default: ox = 0; oy = 1; oz = val; break;
                }
                ev[e] = make_float3((fx + ox) * sv.voxel, (fy + oy) * sv.voxel, (fz + oz) * sv.voxel);
            }
            for (int k = 0; k < t; ++k) {
                const long long tid = first + k;
                if (tid >= max_tris) break;
                const int e0 = (int)((packed >> (4 + 12 * k)) & 0xF);
                const int e1 = (int)((packed >> (8 + 12 * k)) & 0xF);
                const int e2 = (int)((packed >> (12 + 12 * k)) & 0xF);
                const float3 a = ev[e0], bb = ev[e1], c = ev[e2];
                vtx[tid * 3] = a;
                vtx[tid * 3 + 1] = bb;
                vtx[tid * 3 + 2] = c;
                if (mode == GBF_MESH_NORMAL) {
                    const float3 u = make_float3(bb.x - a.x, bb.y - a.y, bb.z - a.z);
                    const float3 v = make_float3(c.x - a.x, c.y - a.y, c.z - a.z);
                    const float3 nn = cross3(u, v);
                    const float l = norm3(nn.x, nn.y, nn.z);
                    const float3 nrm = make_float3(nn.x / l, nn.y / l, nn.z / l);
                    float3 *na = static_cast<float3 *>(attr);
                    na[tid * 3] = nrm;
                    na[tid * 3 + 1] = nrm;
                    na[tid * 3 + 2] = nrm;
                } else if (mode == GBF_MESH_COLOUR) {
                    // edges 0-7 take corner e's colour, 8-11 corner e-8 (scene_mesh.cu:526-549)
                    unsigned char *ca = static_cast<unsigned char *>(attr) + tid * 9;
                    const int es[3] = {e0, e1, e2};
                    for (int q = 0; q < 3; ++q) {
                        const int corner = es[q] < 8 ? es[q] : es[q] - 8;
                        const int cell = cc[corner];
                        ca[q * 3 + 0] = sm.rgb[cell][0];
                        ca[q * 3 + 1] = sm.rgb[cell][1];
                        ca[q * 3 + 2] = sm.rgb[cell][2];
                    }
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace

void launch_mesh(const SessionView *d_sv, const Extent &ex, int layout, int mode, float *vtx, void *attr,
                 long long max_tris, int *counts, cudaStream_t st) {
    const int g = min(max(ex.max_pool, 1), 152 * 4);
    float3 *v3 = reinterpret_cast<float3 *>(vtx);
    if (layout == GBF_VOXEL_REF) mesh_count_kernel<GBF_VOXEL_REF><<<g, kBlockVoxels, 0, st>>>(d_sv, mode, counts);
    else if (layout == GBF_VOXEL_HALF) mesh_count_kernel<GBF_VOXEL_HALF><<<g, kBlockVoxels, 0, st>>>(d_sv, mode, counts);
    else mesh_count_kernel<GBF_VOXEL_SNORM><<<g, kBlockVoxels, 0, st>>>(d_sv, mode, counts);
    mesh_scan_kernel<<<1, 1024, 0, st>>>(d_sv, counts);
    if (layout == GBF_VOXEL_REF)
        mesh_emit_kernel<GBF_VOXEL_REF><<<g, kBlockVoxels, 0, st>>>(d_sv, mode, counts, v3, attr, max_tris);
    else if (layout == GBF_VOXEL_HALF)
        mesh_emit_kernel<GBF_VOXEL_HALF><<<g, kBlockVoxels, 0, st>>>(d_sv, mode, counts, v3, attr, max_tris);
    else
        mesh_emit_kernel<GBF_VOXEL_SNORM><<<g, kBlockVoxels, 0, st>>>(d_sv, mode, counts, v3, attr, max_tris);
}

}  // namespace gbf
