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
// partials in FP64 in CTA order and runs the step on the device: FP64 LDL^T
// solve of the 6x6 system, SE(3) exponential, pose composition, and the
// reference's error-increase / revert / break rules.  No host round trip: the
// reference pays two device->host syncs per iteration (pose_estimator.cu:302-304,
// m_estimator.cu:477-479).  The order of every sum is fixed, so a session's
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
// FP64 6x6 LDL^T with symmetric diagonal pivoting (the documented method of
// Eigen::LDLT used at icp_tracker.cpp:92); zero pivots act as a pseudo-inverse.
__device__ void ldlt_solve6(double A[6][6], const double b[6], double x[6]) {
    int perm[6] = {0, 1, 2, 3, 4, 5};
    double D[6];
    for (int k = 0; k < 6; ++k) {
        int p = k;
        double best = fabs(A[k][k]);
        for (int i = k + 1; i < 6; ++i)
            if (fabs(A[i][i]) > best) { best = fabs(A[i][i]); p = i; }
        if (p != k) {
            for (int j = 0; j < 6; ++j) { double t = A[k][j]; A[k][j] = A[p][j]; A[p][j] = t; }
            for (int i = 0; i < 6; ++i) { double t = A[i][k]; A[i][k] = A[i][p]; A[i][p] = t; }
            int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
        }
        D[k] = A[k][k];
        if (fabs(D[k]) <= DBL_MIN) {
            for (int i = k + 1; i < 6; ++i) A[i][k] = 0.0;
            continue;
        }
        for (int i = k + 1; i < 6; ++i) {
            const double t = A[i][k];
            A[i][k] = t / D[k];
            for (int j = k + 1; j <= i; ++j) A[i][j] -= A[i][k] * A[j][k] * D[k];
            // keep the upper triangle symmetric for the next pivot search / swaps
            for (int j = k + 1; j <= i; ++j) A[j][i] = A[i][j];
        }
    }
    double z[6];
    for (int i = 0; i < 6; ++i) z[i] = b[perm[i]];
    for (int i = 0; i < 6; ++i)
        for (int k = 0; k < i; ++k) z[i] -= A[i][k] * z[k];
    for (int i = 0; i < 6; ++i) z[i] = (fabs(D[i]) > DBL_MIN) ? z[i] / D[i] : 0.0;
    for (int i = 5; i >= 0; --i)
        for (int k = i + 1; k < 6; ++k) z[i] -= A[k][i] * z[k];
    for (int i = 0; i < 6; ++i) x[perm[i]] = z[i];
}

// SE(3) exponential of xi = (rho, phi), translation first (Sophus convention).
__device__ void se3_exp(const double xi[6], double T[12]) {
    const double wx = xi[3], wy = xi[4], wz = xi[5];
    const double th2 = wx * wx + wy * wy + wz * wz;
    const double th = sqrt(th2);
    double A, B, C;
    if (th < 1e-5) {
        A = 1.0 - th2 / 6.0;
        B = 0.5 - th2 / 24.0;
        C = 1.0 / 6.0 - th2 / 120.0;
    } else {
        const double s = sin(th), c = cos(th);
        A = s / th;
        B = (1.0 - c) / th2;
        C = (th - s) / (th2 * th);
    }
    const double W[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    double W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) W2[i * 3 + j] = W[i * 3] * W[j] + W[i * 3 + 1] * W[3 + j] + W[i * 3 + 2] * W[6 + j];
    double V[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double I = (i == j) ? 1.0 : 0.0;
            T[i * 4 + j] = I + A * W[i * 3 + j] + B * W2[i * 3 + j];
            V[i * 3 + j] = I + B * W[i * 3 + j] + C * W2[i * 3 + j];
        }
    for (int i = 0; i < 3; ++i) T[i * 4 + 3] = V[i * 3] * xi[0] + V[i * 3 + 1] * xi[1] + V[i * 3 + 2] * xi[2];
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

// RgbReduction2::find_corresp + compute_jacobian (m_estimator.cu:315-391)
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
    const float ic = interp2(sv.inten[cs][level], K.w, u0, v0);
    const float dx = interp2(sv.gx[level], K.w, u0, v0);
    const float dy = interp2(sv.gy[level], K.w, u0, v0);
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
// A thread adds at most 8 pixels before the warp tree and the FP64 pass over
// the CTAs: the summation error stays at or below that of a Kahan-compensated
// sequential float sum without its 29 compensation registers.
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

// One CTA's partial sums over pixels [cta*1024, cta*1024+1024) of a level.
// The reference frame's vertices, normals and intensities of the tile (36 KB)
// are staged in shared memory with asynchronous 16-byte copies issued by all
// threads at once, so each pixel then waits for a single round trip: the
// gather of the current frame at its projection.  Warps 0-3 accumulate ICP
// rows, warps 4-7 photometric rows (29 sums per thread), each thread 8 pixels
// 128 apart; warp shuffle tree, then a fixed-order pass over the four warps of
// each half.  Writes 58 floats to part.
__device__ __forceinline__ void cta_partial(const SessionView &sv, int level, int rs, int cs, const M34 &T,
                                            float stddev, int cta, int tile, float *part) {
    __shared__ float warp_sums[kReduceThreads / 32][29];
    __shared__ __align__(16) float4 s_v[kCtaPixels];
    __shared__ __align__(16) float4 s_n[kCtaPixels];
    __shared__ __align__(16) float s_i[kCtaPixels];
    const PhotoConst pc = photo_const(stddev);
    const int P = sv.lv[level].w * sv.lv[level].h;
    const int first = cta * tile;  // tile <= kCtaPixels, a multiple of 4 (16-byte aligned copies)
    const int n = min(tile, P - first);
    {
        const float4 *gv = sv.vmap[rs][level] + first, *gn = sv.nmap[rs][level] + first;
        const float *gi = sv.inten[rs][level] + first;
        for (int c = threadIdx.x; c < n; c += kReduceThreads) {
            cp_async16(&s_v[c], gv + c);
            cp_async16(&s_n[c], gn + c);
        }
        // intensities in 16-byte chunks; the last chunk may run up to 3 floats past
        // the image, inside the image's 256-byte-rounded allocation
        for (int c = threadIdx.x; c < (n + 3) / 4; c += kReduceThreads) cp_async16(&s_i[4 * c], gi + 4 * c);
        asm volatile("cp.async.commit_group;\ncp.async.wait_all;\n" ::: "memory");
    }
    __syncthreads();
    const int half = threadIdx.x / kHalfThreads, t = threadIdx.x % kHalfThreads;
    float acc[29];
#pragma unroll
    for (int k = 0; k < 29; ++k) acc[k] = 0.f;
#pragma unroll 2
    for (int i = 0; i < kCtaPixels / kHalfThreads; ++i) {
        const int c = t + i * kHalfThreads;
        if (c >= n) break;
        float row[7];
        const bool ok = half == 0 ? icp_row(sv, level, cs, T, s_v[c], s_n[c], row)
                                  : rgb_row(sv, level, cs, T, pc, s_v[c], s_i[c], row);
        if (ok) accumulate(acc, row);
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

// Sum of the n partial records in FP64: 4 groups of 64 threads take every
// fourth record in order, then the 4 group sums are added in order.
__device__ __forceinline__ void sum_partials(const float *parts, int n, double *total) {
    __shared__ double grp[4][kPartialStride];
    const int g = threadIdx.x >> 6, k = threadIdx.x & 63;
    if (k < kReduceWidth) {
        double s = 0.0;
#pragma unroll 4
        for (int c = g; c < n; c += 4) s += (double)__ldcg(parts + (size_t)c * kPartialStride + k);
        grp[g][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < kReduceWidth)
        total[threadIdx.x] = ((grp[0][threadIdx.x] + grp[1][threadIdx.x]) + grp[2][threadIdx.x]) + grp[3][threadIdx.x];
    __syncthreads();
}

struct ReduceArgs {
    int level, iter, once;
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
__global__ void __launch_bounds__(kReduceThreads, 4) gn_reduce_kernel(const SessionView *svs, ReduceArgs a) {
    const SessionView &sv = svs[blockIdx.y];
    const int level = a.level;
    if (!session_runs(sv, a) || blockIdx.x >= sv.red_ctas[level]) return;
    TrackState *ts = sv.ts;
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
    const int rs = ts->idx, cs = 1 - ts->idx;
    cta_partial(sv, level, rs, cs, T, stddev_s, blockIdx.x, sv.red_tile[level],
                sv.partials + (size_t)blockIdx.x * kPartialStride);
    __threadfence();
    __syncthreads();
    __shared__ unsigned int ticket;
    if (threadIdx.x == 0) ticket = atomicAdd(reinterpret_cast<unsigned *>(sv.ctr + C_TICKET), 1u);
    __syncthreads();
    if (ticket != (unsigned)sv.red_ctas[level] - 1u) return;
    __threadfence();
    __shared__ double total[kReduceWidth];
    sum_partials(sv.partials, sv.red_ctas[level], total);
    if (threadIdx.x < kReduceWidth) ts->last_sums[threadIdx.x] = total[threadIdx.x];
    if (threadIdx.x == 0) {
        sv.ctr[C_TICKET] = 0;
        if (!a.once) gn_epilogue(sv, level, a.iter, total);
    }
}

// Host loop body of DenseTracking::compute_transform (icp_tracker.cpp:52-139).
__device__ void gn_epilogue(const SessionView &sv, int level, int iter, const double *s) {
    TrackState *ts = sv.ts;
    // create_jtjjtr (reduce_sum.h:48-61): float matrices from the sums
    float Hi[6][6], Hr[6][6], bi[6], br[6];
    int k = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 7; ++j, ++k) {
            const float vi = (float)s[k], vr = (float)s[29 + k];
            if (j == 6) {
                bi[i] = vi; br[i] = vr;
            } else {
                Hi[i][j] = Hi[j][i] = vi;
                Hr[i][j] = Hr[j][i] = vr;
            }
        }
    const float r_icp = (float)s[27], n_icp = (float)s[28];
    const float r_rgb = (float)s[29 + 27], n_rgb = (float)s[29 + 28];
    const float stddev_next = sqrtf(r_rgb / (n_rgb - 6.0f));
    double A[6][6], b[6], xi[6];
    for (int i = 0; i < 6; ++i) {
        for (int j = 0; j < 6; ++j) A[i][j] = (double)(sv.w_icp * Hi[i][j] + sv.w_rgb * Hr[i][j]);
        b[i] = (double)(sv.w_icp * bi[i] + sv.w_rgb * br[i]);
    }
    ldlt_solve6(A, b, xi);
    double E[12], next[12];
    se3_exp(xi, E);
    pose_mul(E, ts->est, next);
    pose_copy(ts->est, ts->est_prev);
    pose_copy(next, ts->est);
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
__global__ void track_begin_kernel(const SessionView *svs, int frame_mode) {
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
__global__ void track_finish_kernel(const SessionView *svs, int frame_mode) {
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

int track_launches(int nslots, const Extent &ex) {
    int it = 0;
    for (int l = 0; l < ex.levels; ++l) it += ex.max_iter[l];
    return 2 + ((nslots + kTrackSubgroup - 1) / kTrackSubgroup) * it;
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
                gn_reduce_kernel<<<dim3(ex.max_red[level], n), kReduceThreads, 0, st>>>(d_sv + s0, a);
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
__global__ void slot_results_kernel(const SessionView *svs, int n, gbf_slot_result *out) {
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
// Some callers cannot allocate device memory at all: code running while a CUDA
// graph is being captured (cudaMalloc is not capturable), real-time loops that
// forbid allocation after start-up, and host frameworks that hand out every
// byte of device memory through their own allocator.  For them this entry
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
    __shared__ M34 T;
    if (threadIdx.x == 0)
#pragma unroll
        for (int i = 0; i < 12; ++i) T.m[i] = a.pose[i];
    __syncthreads();
    cta_partial(sv, 0, 0, 1, T, a.stddev, blockIdx.x, kCtaPixels, scratch + (size_t)blockIdx.x * kPartialStride);
    __threadfence();
    __syncthreads();
    __shared__ unsigned int ticket;
    unsigned *tk = reinterpret_cast<unsigned *>(scratch + kStaticTicketSlot);
    if (threadIdx.x == 0) ticket = atomicAdd(tk, 1u);
    __syncthreads();
    if (ticket != (unsigned)nctas - 1u) return;
    __threadfence();
    __shared__ double total[kReduceWidth];
    sum_partials(scratch, nctas, total);
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
