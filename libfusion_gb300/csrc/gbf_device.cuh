// gbf_device.cuh -- device helpers shared by the kernels.
//
// Arithmetic follows the reference's expression order exactly; the library is
// compiled with -fmad=false so that no multiply-add is contracted and every
// float operation rounds as written (the oracle uses -ffp-contract=off).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbf_types.h"
#include "../../include/gbfusion.h"

namespace gbf {

// ---------------------------------------------------------------------------
// float 3x4 rigid transform, rows (R0|t0), (R1|t1), (R2|t2)
// Matrix3x4::operator()(Vector3) (include/math/matrix_type.h:96-100): each row
// is a Vector4 dot with (x, y, z, 1), summed left to right.
struct M34 {
    float m[12];
    __device__ __forceinline__ float3 apply(float x, float y, float z) const {
        return make_float3(((m[0] * x + m[1] * y) + m[2] * z) + m[3] * 1.0f,
                           ((m[4] * x + m[5] * y) + m[6] * z) + m[7] * 1.0f,
                           ((m[8] * x + m[9] * y) + m[10] * z) + m[11] * 1.0f);
    }
    // Matrix3x4::rotate (matrix_type.h:88-94)
    __device__ __forceinline__ float3 rotate(float x, float y, float z) const {
        return make_float3((m[0] * x + m[1] * y) + m[2] * z,
                           (m[4] * x + m[5] * y) + m[6] * z,
                           (m[8] * x + m[9] * y) + m[10] * z);
    }
};

__device__ __forceinline__ M34 pose_to_float(const double *p) {
    M34 r;
#pragma unroll
    for (int i = 0; i < 12; ++i) r.m[i] = (float)p[i];
    return r;
}

// SE3 inverse in double: (R^T, -(R^T t)); sums left to right.
__device__ __forceinline__ void pose_inverse(const double *p, double *o) {
    o[0] = p[0]; o[1] = p[4]; o[2] = p[8];
    o[4] = p[1]; o[5] = p[5]; o[6] = p[9];
    o[8] = p[2]; o[9] = p[6]; o[10] = p[10];
    o[3] = -((o[0] * p[3] + o[1] * p[7]) + o[2] * p[11]);
    o[7] = -((o[4] * p[3] + o[5] * p[7]) + o[6] * p[11]);
    o[11] = -((o[8] * p[3] + o[9] * p[7]) + o[10] * p[11]);
}

// c = a * b
__device__ __forceinline__ void pose_mul(const double *a, const double *b, double *c) {
    double r[12];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r[i * 4 + j] = (a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j]) + a[i * 4 + 2] * b[2 * 4 + j];
        r[i * 4 + 3] = ((a[i * 4 + 0] * b[3] + a[i * 4 + 1] * b[7]) + a[i * 4 + 2] * b[11]) + a[i * 4 + 3];
    }
#pragma unroll
    for (int i = 0; i < 12; ++i) c[i] = r[i];
}

__device__ __forceinline__ void pose_identity(double *p) {
#pragma unroll
    for (int i = 0; i < 12; ++i) p[i] = (i == 0 || i == 5 || i == 10) ? 1.0 : 0.0;
}

__device__ __forceinline__ void pose_copy(const double *a, double *b) {
#pragma unroll
    for (int i = 0; i < 12; ++i) b[i] = a[i];
}

// float forms of the mapping pose, computed once whenever map_pose changes
__device__ __forceinline__ void update_map_floats(TrackState *ts) {
    double inv[12];
    pose_inverse(ts->map_pose, inv);
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        ts->map_twc[i] = (float)ts->map_pose[i];
        ts->map_tcw[i] = (float)inv[i];
    }
}

__device__ __forceinline__ M34 load_m34(const float *m) {
    M34 r;
#pragma unroll
    for (int i = 0; i < 12; ++i) r.m[i] = m[i];
    return r;
}

// ---------------------------------------------------------------------------
// a / b rounded to nearest, from y = 1/b rounded to nearest (__frcp_rn): the
// quotient a*y corrected twice by the exact remainder r = a - b*q (one fused
// multiply-add).  The first correction leaves q within one unit in the last
// place of a/b; from such a q and the correctly rounded y, the second gives
// the correctly rounded quotient (Markstein's theorem: P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990; also in J.-M. Muller et al., Handbook of Floating-Point
// Arithmetic, on division with a fused multiply-add), barring overflow and
// underflow.  Callers that share b between several quotients compute y once.
// Used for the integration's four running means, which share b (|a| <= 255 *
// 510, 0 < b <= 510, nonzero |a / b| far above the subnormal range; a is never
// -0 there, which would need both products -0, so a zero quotient keeps its
// sign; tests/test_arith_proofs.py checks the steps in exact arithmetic on these
// ranges).  For two quotients sharing b (the voxel and photometric
// projections) it measured slower than two divisions.
__device__ __forceinline__ float div_rn_by(float a, float b, float y) {
    const float q0 = __fmul_rn(a, y);
    const float q1 = __fmaf_rn(__fmaf_rn(-q0, b, a), y, q0);
    return __fmaf_rn(__fmaf_rn(-q1, b, a), y, q1);
}

// Vector3 helpers in the reference's order (include/math/vector_type.h)
__device__ __forceinline__ float norm3(float x, float y, float z) {
    return sqrtf((x * x + y * y) + z * z);
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// ToVector3i (vector_type.h:218-225): truncate, then step down when above --
// floor(v), one round-down conversion.  The two differ only below -2^31, where
// the reference's step down overflows; such positions are outside the map's
// coordinate range either way.
__device__ __forceinline__ int floor_ref(float v) { return __float2int_rd(v); }

// voxelPosToBlockPos (map_struct.cu:626-636): (v < 0 ? v - 7 : v) / 8 with
// truncating division is floor(v / 8), an arithmetic shift
__device__ __forceinline__ int voxel_to_block(int v) { return v >> 3; }
// voxelPosToLocalPos (map_struct.cu:643-655): v % 8, plus 8 when negative = v & 7
__device__ __forceinline__ int voxel_to_local(int v) { return v & 7; }

// computeHash (map_struct.cu:143-148) with defined 32-bit wraparound.
__host__ __device__ __forceinline__ int compute_hash(int x, int y, int z, int n) {
    unsigned ux = (unsigned)x * 73856093u, uy = (unsigned)y * 19349669u, uz = (unsigned)z * 83492791u;
    int res = (int)(ux ^ uy ^ uz);
    res %= n;
    return res < 0 ? res + n : res;
}

__host__ __device__ __forceinline__ unsigned long long pack_key(int x, int y, int z) {
    const unsigned long long m = (1ull << kCoordBits) - 1ull;
    return (((unsigned long long)(unsigned)x & m) << (2 * kCoordBits)) |
           (((unsigned long long)(unsigned)y & m) << kCoordBits) | ((unsigned long long)(unsigned)z & m);
}

__device__ __forceinline__ bool coord_ok(int x, int y, int z) {
    return x > -kCoordLimit && x < kCoordLimit && y > -kCoordLimit && y < kCoordLimit && z > -kCoordLimit &&
           z < kCoordLimit;
}

// Home slot: computeHash modulo the slot count; for a power-of-two count the
// non-negative remainder is the low bits.
// Lookups take any view with the SessionView field names they read (table,
// cap, cap_mask, max_probe): the session itself, or a copy of those fields a
// kernel keeps in registers.
template <class SV>
__device__ __forceinline__ int home_slot(const SV &sv, int x, int y, int z) {
    if (sv.cap_mask >= 0) {
        const unsigned ux = (unsigned)x * 73856093u, uy = (unsigned)y * 19349669u, uz = (unsigned)z * 83492791u;
        return (int)((ux ^ uy ^ uz) & (unsigned)sv.cap_mask);
    }
    return compute_hash(x, y, z, sv.cap);
}

// Read-only lookup: pool block id or -1.
template <class SV>
__device__ __forceinline__ int find_block(const SV &sv, int bx, int by, int bz) {
    if (!coord_ok(bx, by, bz)) return -1;
    const unsigned long long key = pack_key(bx, by, bz);
    int slot = home_slot(sv, bx, by, bz);
    for (int p = 0; p < sv.max_probe; ++p) {
        const int4 e = __ldg(reinterpret_cast<const int4 *>(sv.table) + slot);
        const unsigned long long k = ((unsigned long long)(unsigned)e.y << 32) | (unsigned)e.x;
        if (k == key) return e.z;
        if (k == kEmptyKey) return -1;
        slot = (slot + 1 == sv.cap) ? 0 : slot + 1;
    }
    return -1;
}

// ---------------------------------------------------------------------------
// Voxel storage.  REF: int16 sdf packed as (short)(v*32767) (truncation),
// unpacked as v/32767.f; float weight clamped to 255 (include/data_struct/
// voxel.h:36-66).  HALF: fp16 sdf and fp16 weight (clamped to 255), both
// rounded to nearest.  SNORM: int16 sdf packed as v*32767 rounded to nearest and
// unpacked by one multiply with kSnormUnit, and HALF's fp16 weight.  HALF and
// SNORM keep sdf (low 16 bits) and weight (high 16 bits) in one 32-bit word.
struct Vox {
    float sdf;
    float w;
    uchar4 rgb;
};

// v / 32767.f correctly rounded (Voxel::getSDF, voxel.h:36-39) without a
// division: q = v * RN(1/32767), then one correction with the exact residual
// v - q * 32767 (Markstein's method; P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990).  Equal to the division for all 65,535 int16 codes (checked with exact
// rational arithmetic, tests/test_arith_proofs.py).
constexpr float kRefUnitRN = 1.0f / 32767.0f;  // RN(1/32767), evaluated at compile time
__device__ __forceinline__ float sdf_ref_unpack(short v) {
    const float x = (float)v;
    const float q = x * kRefUnitRN;
    const float e = __fmaf_rn(-q, 32767.f, x);
    return __fmaf_rn(e, kRefUnitRN, q);
}
__device__ __forceinline__ short sdf_ref_pack(float v) { return (short)__float2int_rz(v * 32767.f); }
__device__ __forceinline__ float weight_ref_store(float w) { return w > 255.f ? 255.f : w; }
// HALF weight: the clamped float weight rounded to binary16 (11-bit significand,
// range to 65504).  A linear 16-bit code over [0, 255] would quantise one
// observation's weight (|sin n_z| / d^2, often below 0.1) by several percent.
__device__ __forceinline__ unsigned short weight_half_pack(float w) {
    return __half_as_ushort(__float2half_rn(w > 255.f ? 255.f : w));
}
__device__ __forceinline__ float weight_half_unpack(unsigned short q) { return __half2float(__ushort_as_half(q)); }

// SNORM unit: the float just above 1/32767 (1/32767 rounded up).  A multiply
// replaces REF's divide, and because code * kSnormUnit * 32767 >= code for every
// int16 code, both the truncating REF pack (a map dump) and the rounding SNORM
// pack return the code unchanged.  |sdf| reaches 1 + 2^-23 at code +-32767.
constexpr float kSnormUnit = 0x1.000202p-15f;

// sdf code of the 32-bit word layouts
template <int LAYOUT>
__device__ __forceinline__ float sdf_word_unpack(unsigned short code) {
    if (LAYOUT == GBF_VOXEL_HALF) return __half2float(__ushort_as_half(code));
    return (float)(short)code * kSnormUnit;
}
template <int LAYOUT>
__device__ __forceinline__ unsigned sdf_word_pack(float v) {
    if (LAYOUT == GBF_VOXEL_HALF) return (unsigned)__half_as_ushort(__float2half_rn(v));
    return (unsigned)(unsigned short)(short)__float2int_rn(v * 32767.f);
}

// One load gives sdf and weight: HALF packs them in a 32-bit word, REF in 64 bits.
template <int LAYOUT>
__device__ __forceinline__ float unpack_sw(unsigned lo, unsigned hi, float &w) {
    if (LAYOUT == GBF_VOXEL_REF) {
        w = __uint_as_float(hi);
        return sdf_ref_unpack((short)(lo & 0xffffu));
    } else {
        w = weight_half_unpack((unsigned short)(lo >> 16));
        return sdf_word_unpack<LAYOUT>((unsigned short)(lo & 0xffffu));
    }
}

// load_vox / store_sw on explicit pool pointers (no descriptor reads)
template <int LAYOUT>
__device__ __forceinline__ Vox load_vox_at(const void *__restrict__ sw, const uchar4 *__restrict__ rgb, int i) {
    Vox v;
    if (LAYOUT == GBF_VOXEL_REF) {
        const uint2 q = reinterpret_cast<const uint2 *>(sw)[i];
        v.sdf = unpack_sw<LAYOUT>(q.x, q.y, v.w);
    } else {
        const unsigned q = reinterpret_cast<const unsigned *>(sw)[i];
        v.sdf = unpack_sw<LAYOUT>(q, 0u, v.w);
    }
    v.rgb = rgb[i];
    return v;
}
template <int LAYOUT>
__device__ __forceinline__ void store_sw_at(void *__restrict__ sw, int i, float sdf, float w) {
    if (LAYOUT == GBF_VOXEL_REF)
        reinterpret_cast<uint2 *>(sw)[i] =
            make_uint2((unsigned)(unsigned short)sdf_ref_pack(sdf), __float_as_uint(weight_ref_store(w)));
    else
        reinterpret_cast<unsigned *>(sw)[i] =
            sdf_word_pack<LAYOUT>(sdf) | ((unsigned)weight_half_pack(w) << 16);
}

template <int LAYOUT>
__device__ __forceinline__ Vox load_vox(const SessionView &sv, size_t i) {
    Vox v;
    if (LAYOUT == GBF_VOXEL_REF) {
        const uint2 q = reinterpret_cast<const uint2 *>(sv.vox_sw)[i];
        v.sdf = unpack_sw<LAYOUT>(q.x, q.y, v.w);
    } else {
        const unsigned q = reinterpret_cast<const unsigned *>(sv.vox_sw)[i];
        v.sdf = unpack_sw<LAYOUT>(q, 0u, v.w);
    }
    v.rgb = sv.vox_rgb[i];
    return v;
}

// sdf + weight through the read-only path (raycast / meshing).  Weight zero = unobserved.
template <int LAYOUT>
__device__ __forceinline__ float load_sdf(const SessionView &sv, size_t i, float &w) {
    if (LAYOUT == GBF_VOXEL_REF) {
        const uint2 q = __ldg(reinterpret_cast<const uint2 *>(sv.vox_sw) + i);
        return unpack_sw<LAYOUT>(q.x, q.y, w);
    } else {
        const unsigned q = __ldg(reinterpret_cast<const unsigned *>(sv.vox_sw) + i);
        return unpack_sw<LAYOUT>(q, 0u, w);
    }
}

// store sdf + weight with the layout's quantisation (voxel.h:36-66 for REF)
template <int LAYOUT>
__device__ __forceinline__ void store_sw(const SessionView &sv, size_t i, float sdf, float w) {
    if (LAYOUT == GBF_VOXEL_REF) {
        reinterpret_cast<uint2 *>(sv.vox_sw)[i] =
            make_uint2((unsigned)(unsigned short)sdf_ref_pack(sdf), __float_as_uint(weight_ref_store(w)));
    } else {
        reinterpret_cast<unsigned *>(sv.vox_sw)[i] =
            sdf_word_pack<LAYOUT>(sdf) | ((unsigned)weight_half_pack(w) << 16);
    }
}

// ---------------------------------------------------------------------------
// status bits
__device__ __forceinline__ void raise_flag(const SessionView &sv, unsigned bits) {
    atomicOr(reinterpret_cast<unsigned *>(sv.ctr + C_STATUS), bits);
}

// warp-aggregated append: returns this lane's index in dst (all active lanes with pred).
__device__ __forceinline__ int warp_append(int *counter, bool pred) {
    const unsigned mask = __activemask();
    const unsigned ballot = __ballot_sync(mask, pred);
    if (!ballot) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return pred ? base + __popc(ballot & ((1u << lane) - 1u)) : -1;
}

// Insert (or find) one block in the session table; stamps it with `frame`.
__device__ __forceinline__ int insert_block(const SessionView &sv, unsigned long long key, int bx, int by, int bz, int frame) {
    int slot = home_slot(sv, bx, by, bz);
    for (int p = 0; p < sv.max_probe; ++p) {
        HashSlot *e = sv.table + slot;
        unsigned long long k = __ldcg(&e->key);
        if (k == kEmptyKey) {
            k = atomicCAS(&e->key, kEmptyKey, key);
            if (k == kEmptyKey) {
                // this thread owns the new slot: take a pool block
                const int id = atomicAdd(sv.ctr + C_NUSED, 1);
                if (id < sv.pool) {
                    sv.bcoord[id] = make_int4(bx, by, bz, slot);
                    sv.bstamp[id] = frame;
                    sv.bfresh[id] = 1;
                    __stcg(&e->ptr, id);
                    return id;
                }
                raise_flag(sv, GBF_FLAG_POOL_EXHAUSTED);
                return -1;
            }
        }
        if (k == key) {
            // existing block; a concurrent creator stamps its own block, so a
            // pending (-1) id needs no wait
            const int id = __ldcg(&e->ptr);
            if (id >= 0) sv.bstamp[id] = frame;
            return id;
        }
        slot = (slot + 1 == sv.cap) ? 0 : slot + 1;
    }
    raise_flag(sv, GBF_FLAG_HASH_FULL);
    return -1;
}

}  // namespace gbf
