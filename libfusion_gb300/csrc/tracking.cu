// tracking.cu -- fused point-to-plane ICP + photometric normal equations and
// the device-side Gauss-Newton step (src/tracking/pose_estimator.cu:166-307,
// src/tracking/m_estimator.cu:313-482, include/tracking/reduce_sum.h:11-61,
// src/tracking/icp_tracker.cpp:23-156).
//
// GB300 design: one launch per (level, iteration) for all sessions of a batch.
// Each CTA reduces its pixels' ICP row and photometric row (the reference runs
// two kernels, each re-reading the reference vertex map) into 29 + 29 FP32
// sums (warp shuffle tree, then a fixed-order shared-memory pass), writes one
// partial record, and the last CTA of the session (atomic ticket) adds the
// partials in a fixed order by compensated float addition, then its first warp
// runs the step on the device: FP64 LDL^T solve of the 6x6 system, SE(3)
// exponential, pose composition, and the reference's error-increase / revert /
// break rules.  Launches of 32 or more sessions take the sum and the step in a
// launch of their own (one CTA per session) instead, so that the reduction's
// CTAs end without a fence and a ticket; the sums and the step are the same.
// No host round trip: the reference pays two device->host syncs per iteration
// (pose_estimator.cu:302-304, m_estimator.cu:477-479).  The order of every sum is fixed, so a session's
// result does not depend on the other sessions in the batch.
#include <float.h>
#include <string.h>

#include <mutex>

#include "gbf_device.cuh"
#include "gbf_internal.h"
#include "gbf_kernels.h"

namespace gbf {

namespace {

// ---------------------------------------------------------------------------
// The Gauss-Newton step in FP64, spread over one warp: the 6x6 LDL^T with
// symmetric diagonal pivoting (the documented method of Eigen::LDLT used at
// icp_tracker.cpp:92; zero pivots act as a pseudo-inverse), the SE(3)
// exponential of xi = (rho, phi), translation first (Sophus convention), and
// the pose composition.  A dependent FP64 operation takes about 70 cycles on
// this part and a division about 600: one thread doing the step alone took
// ~26 us (and spilled the pivoted matrix to local memory), one warp takes
// ~12 us.  Each value sees the same operations in the same order as in the
// one-thread form (row-by-row elimination, forward and back substitution,
// W^2, I + A W + B W^2 and V), which 4,000 generated cases reproduced bit for
// bit, zero pivots and ties in the pivot search included.

// Full-warp shuffles: every lane must reach each call (none may sit inside a
// lane-dependent branch or operand).
__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ int shfl_i(int v, int src) { return __shfl_sync(0xffffffffu, v, src); }
// lane holding the unordered pair {a, b} of a symmetric 6x6 matrix (lower triangle, 21 lanes)
__device__ __forceinline__ int tri6(int a, int b) { return a >= b ? a * (a + 1) / 2 + b : b * (b + 1) / 2 + a; }
__device__ __forceinline__ int diag6(int a) { return a * (a + 1) / 2 + a; }

// x = A^-1 b.  In: lane tri6(r, c) holds A[r][c] (r >= c) in a,
// lane o < 6 holds b[o] in bv.  Out: lane o < 6 gets x[o].  The symmetric
// pivoting is a permutation the lanes track -- lane q < 6 holds perm[q] (the
// original index at logical position q) and pos[q] (the logical position of
// original index q) -- instead of moving rows and columns.
__device__ double ldlt_solve6_warp(double a, double bv) {
    const int lane = threadIdx.x & 31;
    int r = 0;
    while (r < 5 && (r + 1) * (r + 2) / 2 <= lane) ++r;
    const int c = lane < 21 ? lane - r * (r + 1) / 2 : 0;
    if (lane >= 21) r = 0;
    int perm = lane, pos = lane;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        // the first logical i >= k with the largest |A(i,i)| (strictly larger replaces)
        int p = k;
        double best = fabs(shfl_d(a, diag6(shfl_i(perm, k))));
#pragma unroll
        for (int i = k + 1; i < 6; ++i) {
            const double v = fabs(shfl_d(a, diag6(shfl_i(perm, i))));
            if (v > best) {
                best = v;
                p = i;
            }
        }
        if (p != k) {
            const int ok = shfl_i(perm, k), op = shfl_i(perm, p);
            if (lane == k) perm = op;
            if (lane == p) perm = ok;
            if (lane == ok) pos = p;
            if (lane == op) pos = k;
        }
        const int pk = shfl_i(perm, k);
        const double Dk = shfl_d(a, diag6(pk));
        const int li = shfl_i(pos, r), lj = shfl_i(pos, c);
        const int hi = max(li, lj), lo = min(li, lj);
        const bool mine = lane < 21;
        if (fabs(Dk) <= DBL_MIN) {
            if (mine && lo == k && hi > k) a = 0.0;
            continue;
        }
        if (mine && lo == k && hi > k) a = a / Dk;  // L(hi, k) = A(hi, k) / D(k)
        const double Lh = shfl_d(a, tri6(shfl_i(perm, hi), pk));
        const double Ll = shfl_d(a, tri6(shfl_i(perm, lo), pk));
        if (mine && lo > k) a -= Lh * Ll * Dk;
    }
    // forward: z[i] -= L(i, k) z[k], k ascending; lane q < 6 holds z[q] (logical)
    const int src = lane < 6 ? perm : 0;
    double z = shfl_d(bv, src);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double zk = shfl_d(z, k);
        const int pk = shfl_i(perm, k);  // every lane takes part in every shuffle
        const double L = shfl_d(a, lane < 6 ? tri6(perm, pk) : 0);
        if (lane > k && lane < 6) z -= L * zk;
    }
    {
        const double Dq = shfl_d(a, lane < 6 ? diag6(perm) : 0);
        if (lane < 6) z = (fabs(Dq) > DBL_MIN) ? z / Dq : 0.0;
    }
    // backward: z[i] -= L(k, i) z[k], k = i+1 .. 5 ascending
#pragma unroll
    for (int i = 4; i >= 0; --i) {
        const int pi = shfl_i(perm, i);
        double zi = shfl_d(z, i);
#pragma unroll
        for (int k = i + 1; k < 6; ++k) zi -= shfl_d(a, tri6(shfl_i(perm, k), pi)) * shfl_d(z, k);
        if (lane == i) z = zi;
    }
    return shfl_d(z, lane < 6 ? pos : 0);  // x[perm[q]] = z[q]
}

// element idx of W = [w]x (row-major 3x3)
__device__ __forceinline__ double skew_at(int idx, double wx, double wy, double wz) {
    return idx == 1 ? -wz : idx == 2 ? wy : idx == 3 ? wz : idx == 5 ? -wx : idx == 6 ? -wy : idx == 7 ? wx : 0.0;
}

// T = exp(xi) (lane o < 6 holds xi[o]); lane p < 12 gets T[p] (3x4 row-major).
__device__ double se3_exp_warp(double xi) {
    const int lane = threadIdx.x & 31;
    const double x0 = shfl_d(xi, 0), x1 = shfl_d(xi, 1), x2 = shfl_d(xi, 2);
    const double wx = shfl_d(xi, 3), wy = shfl_d(xi, 4), wz = shfl_d(xi, 5);
    const double th2 = wx * wx + wy * wy + wz * wz;
    const double th = sqrt(th2);
    double A, B, C;
    if (th < 1e-5) {
        const double q = th2 / (lane == 0 ? 6.0 : lane == 1 ? 24.0 : 120.0);
        A = 1.0 - shfl_d(q, 0);
        B = 0.5 - shfl_d(q, 1);
        C = 1.0 / 6.0 - shfl_d(q, 2);
    } else {
        double s, co;
        sincos(th, &s, &co);  // the values of sin(th) and cos(th), one range reduction
        // A = s / th, B = (1 - c) / th^2, C = (th - s) / (th^2 th): three lanes, one division
        const double num = lane == 0 ? s : lane == 1 ? 1.0 - co : th - s;
        const double den = lane == 0 ? th : lane == 1 ? th2 : th2 * th;
        const double q = num / den;
        A = shfl_d(q, 0);
        B = shfl_d(q, 1);
        C = shfl_d(q, 2);
    }
    // lane e < 9: rotation and V element (i, j) = (e / 3, e % 3)
    const int e = lane < 9 ? lane : 0, i = e / 3, j = e % 3;
    const double w2 = skew_at(i * 3, wx, wy, wz) * skew_at(j, wx, wy, wz) +
                      skew_at(i * 3 + 1, wx, wy, wz) * skew_at(3 + j, wx, wy, wz) +
                      skew_at(i * 3 + 2, wx, wy, wz) * skew_at(6 + j, wx, wy, wz);
    const double I = (i == j) ? 1.0 : 0.0, w = skew_at(e, wx, wy, wz);
    const double rot = I + A * w + B * w2;
    const double V = I + B * w + C * w2;
    // lane i < 3: translation V[i] . (x0, x1, x2)
    const int t = lane < 3 ? lane : 0;
    const double tr = shfl_d(V, t * 3) * x0 + shfl_d(V, t * 3 + 1) * x1 + shfl_d(V, t * 3 + 2) * x2;
    // pose layout: lane p = ri * 4 + rj
    const int ri = lane < 12 ? lane / 4 : 0, rj = lane < 12 ? lane % 4 : 0;
    const double rv = shfl_d(rot, ri * 3 + (rj < 3 ? rj : 0));
    const double tv = shfl_d(tr, ri);
    return rj == 3 ? tv : rv;
}

// c = a b (pose_mul) with a spread over the warp (lane p < 12 holds a[p]) and b in
// memory; lane p < 12 gets c[p].
__device__ double pose_mul_warp(double ap, const double *b) {
    const int lane = threadIdx.x & 31;
    const int i = lane < 12 ? lane / 4 : 0, j = lane < 12 ? lane % 4 : 0;
    const double a0 = shfl_d(ap, i * 4), a1 = shfl_d(ap, i * 4 + 1), a2 = shfl_d(ap, i * 4 + 2);
    const double a3 = shfl_d(ap, i * 4 + 3);
    if (j < 3) return (a0 * b[0 * 4 + j] + a1 * b[1 * 4 + j]) + a2 * b[2 * 4 + j];
    return ((a0 * b[3] + a1 * b[7]) + a2 * b[11]) + a3;
}

// |log(T)| of an SE(3) element (the success test, icp_tracker.cpp:145)
__device__ double se3_log_norm(const double T[12]) {
    const double tr = T[0] + T[5] + T[10];
    double c = (tr - 1.0) * 0.5;
    c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
    const double th = acos(c);
    const double vx = T[9] - T[6], vy = T[2] - T[8], vz = T[4] - T[1];
    double k = 0.5;
    const double s = sin(th);
    if (th > 1e-8 && s > 1e-12) k = th / (2.0 * s);
    const double wx = k * vx, wy = k * vy, wz = k * vz;
    // rho = V^-1 t,  V^-1 = I - W/2 + (1/th^2)(1 - A/(2B)) W^2
    const double th2 = wx * wx + wy * wy + wz * wz;
    double f;
    if (th2 < 1e-10) {
        f = 1.0 / 12.0;
    } else {
        const double t = sqrt(th2);
        const double A = sin(t) / t, B = (1.0 - cos(t)) / th2;
        f = (1.0 - A / (2.0 * B)) / th2;
    }
    const double W[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    const double t3[3] = {T[3], T[7], T[11]};
    double rho[3];
    for (int i = 0; i < 3; ++i) {
        double r = t3[i];
        for (int j = 0; j < 3; ++j) {
            double w2 = W[i * 3] * W[j] + W[i * 3 + 1] * W[3 + j] + W[i * 3 + 2] * W[6 + j];
            r += -0.5 * W[i * 3 + j] * t3[j] + f * w2 * t3[j];
        }
        rho[i] = r;
    }
    return sqrt(rho[0] * rho[0] + rho[1] * rho[1] + rho[2] * rho[2] + th2);
}

__device__ __forceinline__ bool finite_pose(const double *T) {
    for (int i = 0; i < 12; ++i)
        if (!isfinite(T[i])) return false;
    return true;
}

// ---------------------------------------------------------------------------
// per-pixel rows
__device__ __forceinline__ float interp2(const float *img, int w, float x, float y) {
    const int u = (int)floorf(x), v = (int)floorf(y);
    const float ax = x - (float)u, ay = y - (float)v;
    const float *r0 = img + (size_t)v * w, *r1 = r0 + w;
    return (r0[u] * (1.0f - ax) + r0[u + 1] * ax) * (1.0f - ay) + (r1[u] * (1.0f - ax) + r1[u + 1] * ax) * ay;
}

// interp2 of the intensity and both gradients at once from the packed
// (I, dI/dx, dI/dy, 0) image: four 16-byte taps, each channel the same
// expression as interp2.
__device__ __forceinline__ float3 interp2_igd(const float4 *img, int w, float x, float y) {
    const int u = (int)floorf(x), v = (int)floorf(y);
    const float ax = x - (float)u, ay = y - (float)v;
    const float4 *r0 = img + (size_t)v * w, *r1 = r0 + w;
    const float4 a = r0[u], b = r0[u + 1], c = r1[u], d = r1[u + 1];
    const float bx = 1.0f - ax, by = 1.0f - ay;
    return make_float3((a.x * bx + b.x * ax) * by + (c.x * bx + d.x * ax) * ay,
                       (a.y * bx + b.y * ax) * by + (c.y * bx + d.y * ax) * ay,
                       (a.z * bx + b.z * ax) * by + (c.z * bx + d.z * ax) * ay);
}

// ICPReduction::searchPoint + getRow (pose_estimator.cu:168-222)
__device__ __forceinline__ bool icp_row(const SessionView &sv, int level, int cs, const M34 &T, const float4 vl,
                                        const float4 nl4, float row[7]) {
    const LevelK &K = sv.lv[level];
    if (isnan(vl.x)) return false;
    const float3 vg = T.apply(vl.x, vl.y, vl.z);
    // float invz = 1.0 / vlast_g.z in the reference: a double division rounded to
    // float.  For a float z that equals the correctly rounded float reciprocal
    // (1/z lies at least 2^-49 relative from any 25-bit rounding midpoint, so
    // the double rounding cannot change it), computed without FP64 hardware.
    const float invz = __frcp_rn(vg.z);
    const int u = __float2int_rd(((vg.x * invz) * K.fx + K.cx) + 0.5f);
    const int v = __float2int_rd(((vg.y * invz) * K.fy + K.cy) + 0.5f);
    if (u < 0 || v < 0 || u >= K.w || v >= K.h) return false;
    const int q = v * K.w + u;
    const float4 vc4 = sv.vmap[cs][level][q];
    const float3 ng = T.rotate(nl4.x, nl4.y, nl4.z);
    const float4 nc4 = sv.nmap[cs][level][q];
    const float dist = norm3(vg.x - vc4.x, vg.y - vc4.y, vg.z - vc4.z);
    const float3 cr = cross3(make_float3(nc4.x, nc4.y, nc4.z), ng);
    const float sine = norm3(cr.x, cr.y, cr.z);
    if (!(sine < sv.icp_angle && dist <= sv.icp_dist && !isnan(nc4.x) && !isnan(ng.x))) return false;
    const float3 vxn = cross3(vg, ng);
    row[0] = ng.x; row[1] = ng.y; row[2] = ng.z;
    row[3] = vxn.x; row[4] = vxn.y; row[5] = vxn.z;
    row[6] = dot3(ng, make_float3(vc4.x - vg.x, vc4.y - vg.y, vc4.z - vg.z));
    return true;
}

// Photometric constants of one reduction, evaluated once per CTA in the
// reference's double precision (m_estimator.cu:366-373).
struct PhotoConst {
    float stddev, huber;
    bool normalise, robust;
};
__device__ __forceinline__ PhotoConst photo_const(float stddev) {
    PhotoConst c;
    c.stddev = stddev;
    c.normalise = (double)stddev > 10e-5;
    c.robust = (double)stddev > 10e-6;
    c.huber = (float)(1.345 * (double)stddev);
    return c;
}

// RgbReduction2::find_corresp + compute_jacobian (m_estimator.cu:315-391).
// PACKED: the current frame's intensity and gradients from its packed image
// (sessions); otherwise from the three separate images (caller-owned images).
template <bool PACKED>
__device__ __forceinline__ bool rgb_row(const SessionView &sv, int level, int cs, const M34 &T,
                                        const PhotoConst &pc, const float4 pt, const float il, float row[7]) {
    const float stddev = pc.stddev;
    const LevelK &K = sv.lv[level];
    if (pt.w < 0 || isnan(pt.x)) return false;
    if (!isfinite(il)) return false;
    const float3 q = T.apply(pt.x, pt.y, pt.z);
    const float u0 = (q.x / q.z) * K.fx + K.cx;
    const float v0 = (q.y / q.z) * K.fy + K.cy;
    if (!(u0 >= 2 && u0 < (float)(K.w - 2) && v0 >= 2 && v0 < (float)(K.h - 2))) return false;
    float ic, dx, dy;
    if (PACKED) {
        const float3 g = interp2_igd(sv.igd[cs][level], K.w, u0, v0);
        ic = g.x;
        dx = g.y;
        dy = g.z;
    } else {
        ic = interp2(sv.inten[cs][level], K.w, u0, v0);
        dx = interp2(sv.gx[level], K.w, u0, v0);
        dy = interp2(sv.gy[level], K.w, u0, v0);
    }
    if (!((dx > 2 || dy > 2) && isfinite(ic) && isfinite(dx) && isfinite(dy))) return false;
    const float zi = __frcp_rn(q.z);  // float z_inv = 1.0 / z (same argument as icp_row)
    const float lx = (dx * K.fx) * zi, ly = (dy * K.fy) * zi;
    const float lz = (-(lx * q.x + ly * q.y)) * zi;
    float res = ic - il;
    if (pc.normalise) res /= stddev;
    const float huber = pc.huber;
    float w = 1.f;
    if (fabsf(res) > huber && pc.robust) w = sqrtf(huber / fabsf(res));
    const float3 pl = cross3(q, make_float3(lx, ly, lz));
    row[0] = lx * w; row[1] = ly * w; row[2] = lz * w;
    row[3] = pl.x * w; row[4] = pl.y * w; row[5] = pl.z * w;
    row[6] = w * (-res);
    return true;
}

// The 28 products of the row's upper triangle added into the running sums, one
// fused multiply-add each (the sums are a reduction compared within a
// tolerance, not bit for bit; the rows themselves keep the reference's rounding).
// A thread adds at most 8 pixels before the warp tree and the compensated pass
// over the CTAs: the summation error stays at or below that of a
// Kahan-compensated sequential float sum without its 29 compensation registers.
__device__ __forceinline__ void accumulate(float *acc, const float row[7]) {
    int k = 0;
#pragma unroll
    for (int i = 0; i < 7; ++i)
#pragma unroll
        for (int j = i; j < 7; ++j, ++k) acc[k] = __fmaf_rn(row[i], row[j], acc[k]);
    acc[28] += 1.0f;
}

// Warp sum of 29 per-lane values by recursive halving: at each of the five
// steps a lane keeps half of its values and adds its partner's copy of them
// (xor partner), so the warp moves 31 values per lane instead of 29 x 5.  On
// return lane l (l < 29) holds the warp total of value l.  Fixed pattern:
// deterministic.
template <int N>
__device__ __forceinline__ void halve_step(float (&v)[32], int lane) {
    const bool upper = (lane & N) != 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const float send = upper ? v[i] : v[i + N];
        const float keep = upper ? v[i + N] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, N);
    }
}

__device__ __forceinline__ float warp_sum29(const float (&acc)[29]) {
    const int lane = threadIdx.x & 31;
    float v[32];
#pragma unroll
    for (int k = 0; k < 29; ++k) v[k] = acc[k];
    v[29] = v[30] = v[31] = 0.f;
    halve_step<16>(v, lane);
    halve_step<8>(v, lane);
    halve_step<4>(v, lane);
    halve_step<2>(v, lane);
    halve_step<1>(v, lane);
    return v[0];
}

constexpr int kCtaPixels = kReduceThreads * kReducePixelsPerThread;  // 1024 contiguous pixels per CTA
constexpr int kHalfThreads = kReduceThreads / 2;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

// Shared memory of a reduction CTA.  The last CTA of a session reuses the
// staging tile for the sum of the partial records (sum_partials), so the sum
// costs no shared memory of its own: 8 KB more per CTA measured slower, L1
// (which the projected gathers hit 55% of the time) giving way to it.
struct ReduceSmem {
    float warp_sums[kReduceThreads / 32][29];
    __align__(16) float4 s_v[kCtaPixels];
    __align__(16) float4 s_n[kCtaPixels];
    __align__(16) float s_i[kCtaPixels];
};

// One CTA's partial sums over pixels [cta*1024, cta*1024+1024) of a level.
// The reference frame's vertices, normals and intensities of the tile (36 KB)
// are staged in shared memory with asynchronous 16-byte copies issued at once,
// so each pixel then waits for a single round trip: the gather of the current
// frame at its projection.  Warps 0-3 accumulate ICP rows, warps 4-7
// photometric rows (29 sums per thread), each thread 8 pixels 128 apart; warp
// p and warp p + 4 read the same pixels, so that pair stages them and waits at
// its own 64-thread barrier (staging the whole tile behind the CTA-wide barrier
// measured 1.4% slower over the track phase).  Warp
// shuffle tree, then a fixed-order pass over the four warps of each half.
// Writes 58 floats to part.  The caller issues the tile's copies first
// (stage_ref_tile), so that they are in flight while it loads the pose.
__device__ __forceinline__ void stage_ref_tile(ReduceSmem &sm, const SessionView &sv, int level, int rs, int cta,
                                               int tile) {
    float4 *s_v = sm.s_v, *s_n = sm.s_n;
    float *s_i = sm.s_i;
    const int P = sv.lv[level].w * sv.lv[level].h;
    const int first = cta * tile;  // tile <= kCtaPixels, a multiple of 4 (16-byte aligned copies)
    const int n = min(tile, P - first);
    {
        // Warp p (ICP rows) and warp p + 4 (photometric rows) read the same
        // pixels, c = 128 i + 32 p + lane: the pair stages those alone and meets
        // at its own 64-thread barrier instead of the CTA's.
        const int ln = threadIdx.x & 31, wd = threadIdx.x >> 5, pair = wd & 3;
        const float4 *gv = sv.vmap[rs][level] + first, *gn = sv.nmap[rs][level] + first;
        const float *gi = sv.inten[rs][level] + first;
        if (wd < 4) {  // vertices and normals
#pragma unroll
            for (int i = 0; i < kCtaPixels / kHalfThreads; ++i) {
                const int c = i * kHalfThreads + 32 * pair + ln;
                if (c < n) {
                    cp_async16(&s_v[c], gv + c);
                    cp_async16(&s_n[c], gn + c);
                }
            }
        } else {  // intensities in 16-byte chunks of 4 pixels; a chunk that would run
                  // past the image's last pixel is copied pixel by pixel instead, so
                  // nothing past the image is read
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int q = ln + 32 * j;  // 8 runs of the pair's pixels x 8 chunks
                const int c = (q >> 3) * kHalfThreads + 32 * pair + 4 * (q & 7);
                if (c + 4 <= n) {
                    cp_async16(&s_i[c], gi + c);
                } else {
                    for (int k = c; k < n; ++k) s_i[k] = gi[k];
                }
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
}

template <bool PACKED>
__device__ __forceinline__ void cta_partial(ReduceSmem &sm, const SessionView &sv, int level, int rs, int cs,
                                            const M34 &T, float stddev, int cta, int tile, float *part) {
    auto &warp_sums = sm.warp_sums;
    float4 *s_v = sm.s_v, *s_n = sm.s_n;
    float *s_i = sm.s_i;
    const PhotoConst pc = photo_const(stddev);
    const int P = sv.lv[level].w * sv.lv[level].h;
    const int first = cta * tile;
    const int n = min(tile, P - first);
    {
        // the pair's own copies done, then its 64-thread barrier
        const int pair = (threadIdx.x >> 5) & 3;
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        asm volatile("bar.sync %0, 64;" ::"r"(pair + 1) : "memory");
    }
    const int half = threadIdx.x / kHalfThreads, t = threadIdx.x % kHalfThreads;
    float acc[29];
#pragma unroll
    for (int k = 0; k < 29; ++k) acc[k] = 0.f;
    if (n == kCtaPixels) {
        // a full tile (every CTA but a level's last): a fixed trip count with no
        // bound test lets the compiler overlap one pixel's gathers with the
        // previous pixel's rows (track phase 3.92 -> 3.72 ms against the loop below)
#pragma unroll 2
        for (int i = 0; i < kCtaPixels / kHalfThreads; ++i) {
            const int c = t + i * kHalfThreads;
            float row[7];
            const bool ok = half == 0 ? icp_row(sv, level, cs, T, s_v[c], s_n[c], row)
                                      : rgb_row<PACKED>(sv, level, cs, T, pc, s_v[c], s_i[c], row);
            if (ok) accumulate(acc, row);
        }
    } else {
#pragma unroll 2
        for (int i = 0; i < kCtaPixels / kHalfThreads; ++i) {
            const int c = t + i * kHalfThreads;
            if (c >= n) break;
            float row[7];
            const bool ok = half == 0 ? icp_row(sv, level, cs, T, s_v[c], s_n[c], row)
                                      : rgb_row<PACKED>(sv, level, cs, T, pc, s_v[c], s_i[c], row);
            if (ok) accumulate(acc, row);
        }
    }
    const float total = warp_sum29(acc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane < 29) warp_sums[wid][lane] = total;
    __syncthreads();
    if (lane < 29 && (wid == 0 || wid == 4)) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < 4; ++w) s += warp_sums[wid + w][lane];
        part[(wid == 0 ? 0 : 29) + lane] = s;
    }
}

// Compensated float accumulation: s + c carries the running sum, c the
// rounding errors of the additions, each found exactly by the branch-free
// TwoSum of Knuth (TAOCP vol. 2, 4.2.2) / Moller (1965).  Needs every
// operation rounded as written (no contraction, no reassociation).
struct FSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        const float bp = t - s;
        c += (s - (t - bp)) + (x - bp);
        s = t;
    }
    __device__ __forceinline__ void add(const FSum &o) {
        add(o.s);
        c += o.c;
    }
};

// Sum of the n partial records, in a fixed order, by compensated float
// addition (a single CTA adding thousands of values in FP64 is bound by this
// part's FP64 rate, ~12 us at 300 records): thread t reads the 16-byte chunk
// t % 16 (columns 4(t % 16) .. +3) of records t / 16, t / 16 + 16, ..., then the
// 16 record groups are combined in group order and widened to double.
constexpr int kSumGroups = kReduceThreads / (kPartialStride / 4);  // 16
static_assert(sizeof(float2) * kSumGroups * kPartialStride <= sizeof(float4) * kCtaPixels,
              "the group sums fit in the staging tile");
__device__ __forceinline__ void sum_partials(ReduceSmem &sm, const float *parts, int n, double *total) {
    auto grp = reinterpret_cast<float2 (*)[kPartialStride]>(sm.s_v);  // the tile is dead by now
    const int g = threadIdx.x / (kPartialStride / 4), q = threadIdx.x % (kPartialStride / 4);
    FSum s0, s1, s2, s3;
    const float4 *p4 = reinterpret_cast<const float4 *>(parts) + q;
#pragma unroll 4
    for (int c = g; c < n; c += kSumGroups) {
        const float4 v = __ldcg(p4 + (size_t)c * (kPartialStride / 4));
        s0.add(v.x);
        s1.add(v.y);
        s2.add(v.z);
        s3.add(v.w);
    }
    grp[g][4 * q] = make_float2(s0.s, s0.c);
    grp[g][4 * q + 1] = make_float2(s1.s, s1.c);
    grp[g][4 * q + 2] = make_float2(s2.s, s2.c);
    grp[g][4 * q + 3] = make_float2(s3.s, s3.c);
    __syncthreads();
    if (threadIdx.x < kReduceWidth) {
        FSum t;
#pragma unroll
        for (int h = 0; h < kSumGroups; ++h) {
            const float2 v = grp[h][threadIdx.x];
            FSum o;
            o.s = v.x;
            o.c = v.y;
            t.add(o);
        }
        total[threadIdx.x] = (double)t.s + (double)t.c;
    }
    __syncthreads();
}

struct ReduceArgs {
    int level, iter, once, defer;
    float pose[12];
    float stddev;
};

__device__ void gn_epilogue(const SessionView &sv, int level, int iter, const double *s);

// Whether session `sv` runs this (level, iteration): the schedule of
// compute_transform (icp_tracker.cpp:33-50) with its early `break` per level.
__device__ __forceinline__ bool session_runs(const SessionView &sv, const ReduceArgs &a) {
    if (!sv.active || a.level >= sv.levels) return false;
    if (a.once) return true;
    const TrackState *ts = sv.ts;
    if (!ts->tracking || a.iter >= sv.max_iter[a.level]) return false;
    return !(a.iter > 0 && ts->level_done);
}

// One CTA per (tile, session): the session's sum over 1024 reference pixels
// of the ICP and photometric rows; the CTA that completes the session's last
// tile adds the partials in a fixed order and takes the Gauss-Newton step.
// Sessions that have left the level, or do not track this frame, return at
// once.
__global__ void __launch_bounds__(kReduceThreads, 4) gn_reduce_kernel(const SessionView *__restrict__ svs, ReduceArgs a) {
    const SessionView &sv = svs[blockIdx.y];
    const int level = a.level;
    if (!session_runs(sv, a) || blockIdx.x >= sv.red_ctas[level]) return;
    TrackState *ts = sv.ts;
    const int rs = ts->idx, cs = 1 - rs;
    // the reference tile's copies first: in flight while the pose is loaded
    __shared__ ReduceSmem sm;
    stage_ref_tile(sm, sv, level, rs, blockIdx.x, sv.red_tile[level]);
    __shared__ M34 T;
    __shared__ float stddev_s;
    if (threadIdx.x == 0) {
        if (a.once) {
#pragma unroll
            for (int i = 0; i < 12; ++i) T.m[i] = a.pose[i];
            stddev_s = a.stddev;
        } else {
            T = pose_to_float(ts->est);
            stddev_s = (a.iter == 0) ? 0.f : ts->stddev;
        }
    }
    __syncthreads();
    cta_partial<true>(sm, sv, level, rs, cs, T, stddev_s, blockIdx.x, sv.red_tile[level],
                sv.partials + (size_t)blockIdx.x * kPartialStride);
    if (a.defer) return;  // gn_step_kernel, launched next, sums the partials and takes the step
    __threadfence();
    __syncthreads();
    __shared__ unsigned int ticket;
    if (threadIdx.x == 0) ticket = atomicAdd(reinterpret_cast<unsigned *>(sv.ctr + C_TICKET), 1u);
    __syncthreads();
    if (ticket != (unsigned)sv.red_ctas[level] - 1u) return;
    __threadfence();
    __shared__ double total[kReduceWidth];
    sum_partials(sm, sv.partials, sv.red_ctas[level], total);
    if (threadIdx.x < kReduceWidth) ts->last_sums[threadIdx.x] = total[threadIdx.x];
    if (threadIdx.x == 0) sv.ctr[C_TICKET] = 0;
    if (!a.once && threadIdx.x < 32) gn_epilogue(sv, level, a.iter, total);  // one warp
}

// The session's sum of the partial records and the Gauss-Newton step, as the
// last CTA of gn_reduce_kernel takes them, in a launch of its own (one CTA per
// session) after a deferred reduction: the reduction's CTAs then end without a
// fence and a ticket.
__global__ void __launch_bounds__(kReduceThreads) gn_step_kernel(const SessionView *__restrict__ svs, ReduceArgs a) {
    const SessionView &sv = svs[blockIdx.x];
    if (!session_runs(sv, a)) return;
    __shared__ ReduceSmem sm;
    __shared__ double total[kReduceWidth];
    sum_partials(sm, sv.partials, sv.red_ctas[a.level], total);
    if (threadIdx.x < kReduceWidth) sv.ts->last_sums[threadIdx.x] = total[threadIdx.x];
    if (threadIdx.x < 32) gn_epilogue(sv, a.level, a.iter, total);
}

// Host loop body of DenseTracking::compute_transform (icp_tracker.cpp:52-139),
// run by the 32 lanes of one warp: create_jtjjtr (reduce_sum.h:48-61) into the
// float matrices, A = w_icp H_icp + w_rgb H_rgb and b likewise widened to
// double, the LDL^T solve, T <- exp(xi) T; then lane 0 keeps the books.
__device__ void gn_epilogue(const SessionView &sv, int level, int iter, const double *s) {
    TrackState *ts = sv.ts;
    const int lane = threadIdx.x & 31;
    // lane tri6(r, c) (r >= c): A[r][c]; lane o < 6: b[o].  The packed index of
    // (i, j), i <= j < 7, is 7 i - i (i - 1) / 2 + (j - i).
    double a = 0.0, bv = 0.0;
    {
        int r = 0;
        while (r < 5 && (r + 1) * (r + 2) / 2 <= lane) ++r;
        const int c = lane - r * (r + 1) / 2;  // c <= r
        if (lane < 21) {
            const int k = 7 * c - c * (c - 1) / 2 + (r - c);
            a = (double)(sv.w_icp * (float)s[k] + sv.w_rgb * (float)s[29 + k]);
        }
        if (lane < 6) {
            const int k = 7 * lane - lane * (lane - 1) / 2 + (6 - lane);
            bv = (double)(sv.w_icp * (float)s[k] + sv.w_rgb * (float)s[29 + k]);
        }
    }
    const double xi = ldlt_solve6_warp(a, bv);
    const double E = se3_exp_warp(xi);
    const double next = pose_mul_warp(E, ts->est);
    const double old = lane < 12 ? ts->est[lane] : 0.0;
    __syncwarp();
    if (lane < 12) {
        ts->est_prev[lane] = old;
        ts->est[lane] = next;
    }
    __syncwarp();
    if (lane != 0) return;
    const float r_icp = (float)s[27], n_icp = (float)s[28];
    const float r_rgb = (float)s[29 + 27], n_rgb = (float)s[29 + 28];
    const float stddev_next = sqrtf(r_rgb / (n_rgb - 6.0f));
    ts->iterations += 1;
    ts->level_iters[level] += 1;
    ts->pixel_iterations += (long long)sv.lv[level].w * sv.lv[level].h;
    ts->icp_inliers = n_icp;
    ts->rgb_inliers = n_rgb;

    const float last_icp = (iter == 0) ? FLT_MAX : ts->icp_error;
    const float last_rgb = (iter == 0) ? FLT_MAX : ts->rgb_error;
    int icp_count = (iter == 0) ? 0 : ts->icp_count;
    int rgb_count = (iter == 0) ? 0 : ts->rgb_count;
    ts->level_done = 0;
    ts->stddev = stddev_next;
    float icp_error = sqrtf(r_icp) / n_icp;
    if (isnan(icp_error)) {
        ts->invalid = 1;
        ts->level_done = 1;
        ts->icp_error = icp_error;
        return;
    }
    if (icp_error > last_icp) {
        if (icp_count >= 2) {
            pose_copy(ts->est_prev, ts->est);
            ts->level_done = 1;
            return;
        }
        icp_count++;
        icp_error = last_icp;
    } else {
        icp_count = 0;
    }
    ts->icp_error = icp_error;
    ts->icp_count = icp_count;
    float rgb_error = sqrtf(r_rgb) / n_rgb;
    if (isnan(rgb_error)) {
        ts->invalid = 1;
        ts->level_done = 1;
        ts->rgb_error = rgb_error;
        return;
    }
    if (rgb_error > last_rgb) {
        if (rgb_count >= 2) {
            pose_copy(ts->est_prev, ts->est);
            ts->level_done = 1;
            return;
        }
        rgb_count++;
        rgb_error = last_rgb;
    } else {
        rgb_count = 0;
    }
    ts->rgb_error = rgb_error;
    ts->rgb_count = rgb_count;
}

// frame_mode 1: System frame (track only when a reference exists); 0: gbf_track.
__global__ void track_begin_kernel(const SessionView *__restrict__ svs, int frame_mode) {
    const SessionView &sv = svs[blockIdx.x];
    if (!sv.active || threadIdx.x != 0) return;
    TrackState *ts = sv.ts;
    ts->tracking = frame_mode ? ts->has_ref : 1;
    // Revertable(initial_estimate): curr = init, prev = identity
    pose_copy(ts->init, ts->est);
    pose_identity(ts->est_prev);
    ts->invalid = 0;
    ts->iterations = 0;
    for (int l = 0; l < kMaxLevels; ++l) ts->level_iters[l] = 0;
    ts->level_done = 0;
    ts->icp_error = FLT_MAX;
    ts->rgb_error = FLT_MAX;
    ts->stddev = 0.f;
    ts->icp_count = ts->rgb_count = 0;
    sv.ctr[C_TICKET] = 0;
}

// Tracking result (icp_tracker.cpp:143-155); frame_mode 1 also applies the
// System / DenseOdometry bookkeeping (rgbd_odometry.cpp:39-41): pose update
// and reference swap.
__global__ void track_finish_kernel(const SessionView *__restrict__ svs, int frame_mode) {
    const SessionView &sv = svs[blockIdx.x];
    if (!sv.active || threadIdx.x != 0) return;
    TrackState *ts = sv.ts;
    if (ts->tracking) {
        double inv[12], rel[12];
        pose_inverse(ts->est, inv);
        pose_mul(inv, ts->init, rel);
        const double n = se3_log_norm(rel);
        const bool finite = finite_pose(ts->est);
        const bool fail = ts->invalid || !(n <= 0.1) || !finite;
        if (!finite) raise_flag(sv, GBF_FLAG_NAN_POSE);
        if (fail) {
            pose_identity(ts->update);
            ts->success = 0;
        } else {
            pose_copy(inv, ts->update);
            ts->success = 1;
        }
        if (frame_mode) {
            double np[12];
            pose_mul(ts->pose, ts->update, np);
            pose_copy(np, ts->pose);
            if (fail) raise_flag(sv, GBF_FLAG_TRACK_FAILED);
        }
    } else if (frame_mode) {
        ts->success = 1;
        pose_identity(ts->update);
    }
    if (frame_mode) {
        // the next frame's initial estimate: no motion (the reference), or
        // with the constant-velocity prior the motion this frame tracked
        if (sv.motion_prior && ts->tracking && ts->success)
            pose_inverse(ts->update, ts->init);
        else
            pose_identity(ts->init);
        ts->idx = 1 - ts->idx;
        ts->has_ref = 1;
        pose_copy(ts->pose, ts->map_pose);
        update_map_floats(ts);
        ts->frame_index += 1;
    }
}

}  // namespace

// Sessions whose Gauss-Newton iterations run back to back before the next
// subgroup's: a subgroup's level-0 images (about 25 MB per 640x480 session)
// then stay in L2 from one iteration to the next.
constexpr int kTrackSubgroup = 64;

// Sessions per launch from which the Gauss-Newton step runs as a launch of its
// own (gn_step_kernel) instead of in the last CTA of the reduction: with many
// sessions the reduction's CTAs then end without a fence and a ticket (two
// groups of 32 sessions: track 3.71 -> 3.46 ms, tick 10.85 -> 10.80 ms; of 64:
// 5,950 -> 6,057 frames/s); with fewer, the extra launch per iteration costs
// more than it saves (two groups of 16: 5,764 -> 5,702 frames/s; one session:
// 1,236 -> 1,165 frames/s).
constexpr int kDeferStepSessions = 32;
static bool defer_step(int sessions) { return sessions >= kDeferStepSessions; }

int track_launches(int nslots, const Extent &ex) {
    int it = 0;
    for (int l = 0; l < ex.levels; ++l) it += ex.max_iter[l];
    int n = 0;
    for (int s0 = 0; s0 < nslots; s0 += kTrackSubgroup)
        n += it * (defer_step(min(kTrackSubgroup, nslots - s0)) ? 2 : 1);
    return 2 + n;
}

void launch_track(const SessionView *d_sv, int nslots, const Extent &ex, int frame_mode, cudaStream_t st) {
    track_begin_kernel<<<nslots, 32, 0, st>>>(d_sv, frame_mode);
    ReduceArgs a{};
    a.once = 0;
    for (int s0 = 0; s0 < nslots; s0 += kTrackSubgroup) {
        const int n = min(kTrackSubgroup, nslots - s0);
        for (int level = ex.levels - 1; level >= 0; --level) {
            for (int iter = 0; iter < ex.max_iter[level]; ++iter) {
                a.level = level;
                a.iter = iter;
                a.defer = defer_step(n) ? 1 : 0;
                gn_reduce_kernel<<<dim3(ex.max_red[level], n), kReduceThreads, 0, st>>>(d_sv + s0, a);
                if (a.defer) gn_step_kernel<<<n, kReduceThreads, 0, st>>>(d_sv + s0, a);
            }
        }
    }
    track_finish_kernel<<<nslots, 32, 0, st>>>(d_sv, frame_mode);
}

void launch_reduce_once(const SessionView *d_sv, const Extent &ex, int level, const float *pose12, float stddev,
                        cudaStream_t st) {
    ReduceArgs a{};
    a.once = 1;
    a.level = level;
    a.iter = 0;
    for (int i = 0; i < 12; ++i) a.pose[i] = pose12[i];
    a.stddev = stddev;
    gn_reduce_kernel<<<dim3(ex.max_red[level], 1), kReduceThreads, 0, st>>>(d_sv, a);
}

void launch_frame_finish(const SessionView *d_sv, int nslots, cudaStream_t st) {
    track_finish_kernel<<<nslots, 32, 0, st>>>(d_sv, 1);
}

namespace {
__global__ void slot_results_kernel(const SessionView *__restrict__ svs, int n, gbf_slot_result *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SessionView &sv = svs[i];
    gbf_slot_result r;
    if (!sv.ts) {  // empty slot
        for (int j = 0; j < 16; ++j) r.pose[j] = 0.0;
        r.tracked = 0;
        r.status = 0u;
        r.frame_index = 0;
    } else {
        const TrackState *ts = sv.ts;
        for (int j = 0; j < 12; ++j) r.pose[j] = ts->pose[j];
        r.pose[12] = r.pose[13] = r.pose[14] = 0.0;
        r.pose[15] = 1.0;
        r.tracked = ts->success;
        r.status = (uint32_t)sv.ctr[C_STATUS];
        r.frame_index = ts->frame_index;
    }
    out[i] = r;
}
}  // namespace

void launch_slot_results(const SessionView *d_sv, int nslots, gbf_slot_result *out, cudaStream_t st) {
    slot_results_kernel<<<(nslots + 127) / 128, 128, 0, st>>>(d_sv, nslots, out);
}

}  // namespace gbf

// ============================================================================
// Allocation-free ICP + photometric reduction.
//
// Some callers cannot allocate device memory at all: real-time camera loops
// that forbid allocation once they run (a cudaMalloc can block for
// milliseconds and synchronise the device), and host frameworks that hand out
// every byte of device memory through their own allocator, so that a library
// allocating behind their back would fail or break their accounting.  For them this entry
// point reduces one pyramid level of caller-owned images with no session and no
// cudaMalloc / cudaFree: its per-CTA partial sums and its last-CTA ticket live
// in the file-scope array below, which every GPU that loads the library keeps
// until the process exits.
namespace gbf {
namespace {

constexpr int kStaticReduceCtas = 2048;  // 2048 CTAs x 1024 pixels: up to 2,097,152 pixels per image
constexpr int kStaticTicketSlot = kStaticReduceCtas * kPartialStride;

// partial records of kStaticReduceCtas CTAs, then the ticket (as unsigned bits)
static __device__ __align__(256) float g_reduce_scratch[kStaticTicketSlot + 64];

__global__ void __launch_bounds__(kReduceThreads, 3) reduce_static_kernel(SessionView sv, ReduceArgs a,
                                                                          float *scratch, double *out) {
    const int nctas = sv.red_ctas[0];
    __shared__ ReduceSmem sm;
    stage_ref_tile(sm, sv, 0, 0, blockIdx.x, kCtaPixels);
    __shared__ M34 T;
    if (threadIdx.x == 0)
#pragma unroll
        for (int i = 0; i < 12; ++i) T.m[i] = a.pose[i];
    __syncthreads();
    cta_partial<false>(sm, sv, 0, 0, 1, T, a.stddev, blockIdx.x, kCtaPixels, scratch + (size_t)blockIdx.x * kPartialStride);
    __threadfence();
    __syncthreads();
    __shared__ unsigned int ticket;
    unsigned *tk = reinterpret_cast<unsigned *>(scratch + kStaticTicketSlot);
    if (threadIdx.x == 0) ticket = atomicAdd(tk, 1u);
    __syncthreads();
    if (ticket != (unsigned)nctas - 1u) return;
    __threadfence();
    __shared__ double total[kReduceWidth];
    sum_partials(sm, scratch, nctas, total);
    if (threadIdx.x < kReduceWidth) out[threadIdx.x] = total[threadIdx.x];
    if (threadIdx.x == 0) *tk = 0u;
}

// device address of g_reduce_scratch per device, looked up once with that device current
std::mutex g_scratch_mu;
float *g_scratch_ptr[64] = {};

gbf_status static_scratch(float **ptr) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "gbf_reduce_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(GBF_ERR_INVALID_ARG, "gbf_reduce_noalloc: device index >= 64");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_reduce_scratch);
        if (e != cudaSuccess) return cuda_error(e, "gbf_reduce_noalloc: cudaGetSymbolAddress");
        g_scratch_ptr[dev] = static_cast<float *>(p);
    }
    *ptr = g_scratch_ptr[dev];
    return GBF_OK;
}

}  // namespace
}  // namespace gbf

extern "C" GBF_API gbf_status gbf_reduce_noalloc(const gbf_reduce_inputs *in, const double T[16], float stddev,
                                                 double *out_dev, void *stream) {
    using namespace gbf;
    if (!in || !T || !out_dev || !in->ref_vmap || !in->ref_nmap || !in->ref_intensity || !in->cur_vmap ||
        !in->cur_nmap || !in->cur_intensity || !in->cur_didx || !in->cur_didy)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_reduce_noalloc: null pointer");
    if (in->width < 8 || in->height < 8 || !(in->fx > 0) || !(in->fy > 0))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_reduce_noalloc: bad image size or focal length");
    // the reference images are staged in 16-byte copies, the vertex and normal
    // maps read as float4, the other images as float
    auto aligned = [](const void *p, uintptr_t n) { return reinterpret_cast<uintptr_t>(p) % n == 0; };
    if (!aligned(in->ref_vmap, 16) || !aligned(in->ref_nmap, 16) || !aligned(in->ref_intensity, 16) ||
        !aligned(in->cur_vmap, 16) || !aligned(in->cur_nmap, 16) || !aligned(in->cur_intensity, 4) ||
        !aligned(in->cur_didx, 4) || !aligned(in->cur_didy, 4))
        return set_error(GBF_ERR_INVALID_ARG,
                         "gbf_reduce_noalloc: vertex, normal and reference intensity images must be 16-byte aligned");
    if (!aligned(out_dev, 8))  // written as doubles
        return set_error(GBF_ERR_INVALID_ARG, "gbf_reduce_noalloc: out_dev must be 8-byte aligned");
    const long long pixels = (long long)in->width * in->height;
    if (pixels > (long long)kStaticReduceCtas * kReduceThreads * kReducePixelsPerThread)
        return set_error(GBF_ERR_CAPACITY, "gbf_reduce_noalloc: at most 2,097,152 pixels per image");
    float *scratch = nullptr;
    gbf_status st = static_scratch(&scratch);
    if (st != GBF_OK) return st;
    // a SessionView over the caller's level-0 images: set 0 = reference, set 1 = current
    SessionView sv;
    memset(&sv, 0, sizeof(sv));
    sv.levels = 1;
    LevelK &K = sv.lv[0];
    K.w = in->width; K.h = in->height;
    K.fx = in->fx; K.fy = in->fy; K.cx = in->cx; K.cy = in->cy;
    K.invfx = 1.0f / in->fx; K.invfy = 1.0f / in->fy;
    sv.red_ctas[0] = reduce_ctas((int)pixels);
    sv.icp_dist = in->dist_thresh;
    sv.icp_angle = in->angle_thresh;
    sv.vmap[0][0] = (float4 *)in->ref_vmap;
    sv.nmap[0][0] = (float4 *)in->ref_nmap;
    sv.inten[0][0] = (float *)in->ref_intensity;
    sv.vmap[1][0] = (float4 *)in->cur_vmap;
    sv.nmap[1][0] = (float4 *)in->cur_nmap;
    sv.inten[1][0] = (float *)in->cur_intensity;
    sv.gx[0] = (float *)in->cur_didx;
    sv.gy[0] = (float *)in->cur_didy;
    ReduceArgs a{};
    a.once = 1;
    for (int i = 0; i < 12; ++i) a.pose[i] = (float)T[i];
    a.stddev = stddev;
    cudaStream_t s = (cudaStream_t)stream;
    // the ticket must start at zero whatever an earlier, interrupted call left
    cudaError_t e = cudaMemsetAsync(scratch + kStaticTicketSlot, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return cuda_error(e, "gbf_reduce_noalloc: clear ticket");
    reduce_static_kernel<<<sv.red_ctas[0], kReduceThreads, 0, s>>>(sv, a, scratch, out_dev);
    return check_cuda("gbf_reduce_noalloc");
}
