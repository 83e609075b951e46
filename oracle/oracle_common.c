/*
 * oracle_common.c -- integer helpers and tables shared by both oracle
 * precisions.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

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

/* ---- renderPoint / renderSceneK / renderSceneTexturedK (cuda_imgproc.cu:17-108) ---- */

typedef struct { float x, y, z; } F3;

static F3 f3(float x, float y, float z) { F3 v = {x, y, z}; return v; }
/* Vector3::operator* (dot, vector_type.h:83-86) and norm (:98-101) */
static float f3_dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
/* normalised(V) = V / V.norm() (vector_type.h:198-201) */
static F3 f3_normalised(F3 v) {
    const float n = sqrtf((v.x * v.x + v.y * v.y) + v.z * v.z);
    return f3(v.x / n, v.y / n, v.z / n);
}
/* __saturatef(x) * 255.f, then static_cast<unsigned char> */
static uint8_t sat255(float v) {
    const float s = (v != v) ? 0.f : (v < 0.f ? 0.f : (v > 1.f ? 1.f : v));
    return (uint8_t)(s * 255.f);
}

float or_powf20(float x);

static void render_point(F3 p, F3 n, F3 img, F3 light, uint8_t out[4]) {
    float c0 = 4.f / 255.f, c1 = 2.f / 255.f, c2 = 2.f / 255.f;
    if (!(p.x != p.x)) {
        const float Ka = 0.3f, Kd = 0.5f, Ks = 0.2f, sp = 20.f;
        const float Ax = img.x, Dx = img.y, Sx = img.z, Lx = 1.f;
        const F3 L = f3_normalised(f3(light.x - p.x, light.y - p.y, light.z - p.z));
        const F3 V = f3_normalised(f3(0.f - p.x, 0.f - p.y, 0.f - p.z));
        /* 2 * normal: operator*(T S, Vector3<U> V) with T = int returns Vector3<int>,
         * truncating 2 n to integers (vector_type.h:168-172); then * (normal * L) as float */
        const float nl = f3_dot(n, L);
        const int tx = or_trunc_sat(n.x * 2.f), ty = or_trunc_sat(n.y * 2.f), tz = or_trunc_sat(n.z * 2.f);
        const F3 R = f3_normalised(f3((float)tx * nl - L.x, (float)ty * nl - L.y, (float)tz * nl - L.z));
        const float rv = f3_dot(R, V);
        (void)sp;  /* the exponent, 20: or_powf20 */
        const float Ix = ((Ax * Ka) * Dx + ((Lx * Kd) * Dx) * fmaxf(0.f, nl)) + ((Lx * Ks) * Sx) * or_powf20(fmaxf(0.f, rv));
        c0 = c1 = c2 = Ix;
    }
    out[0] = sat255(c0);
    out[1] = sat255(c1);
    out[2] = sat255(c2);
    out[3] = 255;
}

void or_render_scene(const float *vmap, const float *nmap, const uint8_t *rgb, int w, int h, uint8_t *out) {
    const F3 light = f3(5.f, 5.f, 5.f);
    for (int i = 0; i < w * h; ++i) {
        const F3 p = f3(vmap[4 * i], vmap[4 * i + 1], vmap[4 * i + 2]);
        const F3 n = f3(nmap[4 * i], nmap[4 * i + 1], nmap[4 * i + 2]);
        const F3 img = rgb ? f3((float)rgb[3 * i] / 255.f, (float)rgb[3 * i + 1] / 255.f, (float)rgb[3 * i + 2] / 255.f)
                           : f3(1.f, 1.f, 1.f);
        render_point(p, n, img, light, out + 4 * i);
    }
}

/* Sequential float column sums, plain or with Kahan's compensation
 * (W. Kahan, "Further remarks on reducing truncation errors", CACM 8(1), 1965):
 * the yardsticks the GPU reduction's summation error is compared with. */
void or_sum_f32(const float *terms, long long n, int width, int kahan, double *out) {
    for (int k = 0; k < width; ++k) {
        float s = 0.f, c = 0.f;
        for (long long i = 0; i < n; ++i) {
            const float x = terms[i * width + k];
            if (kahan) {
                const float y = x - c;
                const float t = s + y;
                c = (t - s) - y;
                s = t;
            } else {
                s += x;
            }
        }
        out[k] = (double)s;
    }
}

/* Transcendental tables.  The reference's weighted integration and bilateral
 * filter call CUDA's sinf and expf, whose last bits differ from libm's.  For a
 * bit-for-bit comparison a test may hand the FP32 oracle the device's values
 * for exactly the arguments the oracle evaluates: it records the arguments of
 * one run (or_trans_record), has the device evaluate them, installs the pairs
 * (or_trans_table) and runs again.  Every other operation stays the oracle's
 * own; an argument missing from an installed table falls back to libm and is
 * counted (or_trans_misses).  Kind 0: sinf, kind 1: expf, kind 2: powf(x, 20)
 * (the shading's specular term). */
typedef struct {
    uint32_t *x;  /* argument bit patterns, ascending */
    float *y;
    long long n;
    long long misses;
} OrTransTable;
#define OR_TRANS_KINDS 3
static OrTransTable g_trans[OR_TRANS_KINDS];
static uint32_t *g_rec[OR_TRANS_KINDS];
static long long g_rec_n[OR_TRANS_KINDS], g_rec_cap[OR_TRANS_KINDS];
static int g_recording;

static uint32_t f2u(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}

static float trans_eval(int kind, float x) {
    if (g_recording) {
#pragma omp critical(or_trans_record)
        {
            if (g_rec_n[kind] == g_rec_cap[kind]) {
                const long long cap = g_rec_cap[kind] ? 2 * g_rec_cap[kind] : 1 << 16;
                uint32_t *p = (uint32_t *)realloc(g_rec[kind], (size_t)cap * sizeof(uint32_t));
                if (p) {
                    g_rec[kind] = p;
                    g_rec_cap[kind] = cap;
                }
            }
            if (g_rec_n[kind] < g_rec_cap[kind]) g_rec[kind][g_rec_n[kind]++] = f2u(x);
        }
    }
    const OrTransTable *t = &g_trans[kind];
    if (t->n > 0) {
        const uint32_t key = f2u(x);
        long long lo = 0, hi = t->n - 1;
        while (lo <= hi) {
            const long long mid = (lo + hi) / 2;
            if (t->x[mid] == key) return t->y[mid];
            if (t->x[mid] < key) lo = mid + 1;
            else hi = mid - 1;
        }
#pragma omp atomic
        g_trans[kind].misses++;
    }
    return kind == 0 ? sinf(x) : kind == 1 ? expf(x) : powf(x, 20.f);
}

float or_sinf(float x) { return trans_eval(0, x); }
float or_expf(float x) { return trans_eval(1, x); }
float or_powf20(float x) { return trans_eval(2, x); }

/* enable: clear the recorded arguments and start recording; 0: stop (they are kept) */
void or_trans_record(int enable) {
    if (enable)
        for (int k = 0; k < OR_TRANS_KINDS; ++k) g_rec_n[k] = 0;
    g_recording = enable ? 1 : 0;
}

long long or_trans_recorded(int kind, uint32_t *out, long long cap) {
    if (kind < 0 || kind >= OR_TRANS_KINDS) return -1;
    if (out) memcpy(out, g_rec[kind], (size_t)(cap < g_rec_n[kind] ? cap : g_rec_n[kind]) * sizeof(uint32_t));
    return g_rec_n[kind];
}

/* x ascending (unique bit patterns); n = 0 removes the table */
void or_trans_table(int kind, const uint32_t *x, const float *y, long long n) {
    if (kind < 0 || kind >= OR_TRANS_KINDS) return;
    OrTransTable *t = &g_trans[kind];
    free(t->x);
    free(t->y);
    t->x = NULL;
    t->y = NULL;
    t->n = 0;
    t->misses = 0;
    if (n <= 0) return;
    t->x = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    t->y = (float *)malloc((size_t)n * sizeof(float));
    if (!t->x || !t->y) return;
    memcpy(t->x, x, (size_t)n * sizeof(uint32_t));
    memcpy(t->y, y, (size_t)n * sizeof(float));
    t->n = n;
}

long long or_trans_misses(int kind) { return (kind >= 0 && kind < OR_TRANS_KINDS) ? g_trans[kind].misses : -1; }
