/*
 * oracle_impl.h -- body of the CPU oracle, compiled twice: R = float
 * (oracle_f32.c, reference operation order, -ffp-contract=off, quantised voxel
 * storage) and R = double (oracle_f64.c, unquantised storage).
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Every function cites the
 * reference kernel it restates (paths relative to the reference project).
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"

int or_trunc_sat(double v);

#if OR_F64
typedef double R;
#define SFX(n) n##_f64
#define RSQRT sqrt
#define RSIN sin
#define REXP exp
#define RFABS fabs
#define RFLOOR floor
#define RCEIL ceil
#define RFMIN fmin
#define RFMAX fmax
/* (float)(1.0 / (double)x) in the reference; exact division here */
#define INV_D(x) (1.0 / (x))
#define TO_R(x) ((double)(x))
#define HUBER_TH(s) (1.345 * (s))
#else
typedef float R;
#define SFX(n) n##_f32
#define RSQRT sqrtf
#define RSIN or_sinf
#define REXP or_expf
#define RFABS fabsf
#define RFLOOR floorf
#define RCEIL ceilf
#define RFMIN fminf
#define RFMAX fmaxf
#define INV_D(x) ((float)(1.0 / (double)(x)))
#define TO_R(x) ((float)(x))
#define HUBER_TH(s) ((float)(1.345 * (double)(s)))
#endif

typedef struct { R x, y, z; } V3;
typedef struct { R x, y, z, w; } V4;
typedef struct { R m[12]; } M34;

static inline V3 v3(R x, R y, R z) { V3 v = {x, y, z}; return v; }

/* Matrix3x4::operator()(Vector3) (include/math/matrix_type.h:96-100) */
static inline V3 m_apply(const M34 *T, R x, R y, R z) {
    return v3(((T->m[0] * x + T->m[1] * y) + T->m[2] * z) + T->m[3] * (R)1,
              ((T->m[4] * x + T->m[5] * y) + T->m[6] * z) + T->m[7] * (R)1,
              ((T->m[8] * x + T->m[9] * y) + T->m[10] * z) + T->m[11] * (R)1);
}
/* Matrix3x4::rotate (matrix_type.h:88-94) */
static inline V3 m_rotate(const M34 *T, R x, R y, R z) {
    return v3((T->m[0] * x + T->m[1] * y) + T->m[2] * z, (T->m[4] * x + T->m[5] * y) + T->m[6] * z,
              (T->m[8] * x + T->m[9] * y) + T->m[10] * z);
}
/* Vector3::norm / cross / dot (include/math/vector_type.h:98-112) */
static inline R n3(R x, R y, R z) { return RSQRT((x * x + y * y) + z * z); }
static inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline R dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

static inline int floor_r(R v) {
    int b = or_trunc_sat(v);
    return ((R)b > v) ? b - 1 : b;
}
static inline int floor_rd(R v) { return or_trunc_sat(RFLOOR(v)); } /* __float2int_rd */
static inline int vtob(int v) { return (v < 0 ? v - 7 : v) / 8; }
static inline int vtol(int v) { int r = v % 8; return r < 0 ? r + 8 : r; }

/* double SE3 helpers: 3x4 row-major */
static void pose_inv(const double *p, double *o) {
    o[0] = p[0]; o[1] = p[4]; o[2] = p[8];
    o[4] = p[1]; o[5] = p[5]; o[6] = p[9];
    o[8] = p[2]; o[9] = p[6]; o[10] = p[10];
    o[3] = -((o[0] * p[3] + o[1] * p[7]) + o[2] * p[11]);
    o[7] = -((o[4] * p[3] + o[5] * p[7]) + o[6] * p[11]);
    o[11] = -((o[8] * p[3] + o[9] * p[7]) + o[10] * p[11]);
}
static void pose_mul(const double *a, const double *b, double *c) {
    double r[12];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) r[i * 4 + j] = (a[i * 4] * b[j] + a[i * 4 + 1] * b[4 + j]) + a[i * 4 + 2] * b[8 + j];
        r[i * 4 + 3] = ((a[i * 4] * b[3] + a[i * 4 + 1] * b[7]) + a[i * 4 + 2] * b[11]) + a[i * 4 + 3];
    }
    memcpy(c, r, sizeof(r));
}
static void pose_eye(double *p) {
    for (int i = 0; i < 12; ++i) p[i] = (i == 0 || i == 5 || i == 10) ? 1.0 : 0.0;
}
static M34 to_m(const double *p) {
    M34 m;
    for (int i = 0; i < 12; ++i) m.m[i] = TO_R(p[i]);
    return m;
}

static void set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

/* ======================================================================== map */

struct SFX(or_map) {
    or_config cfg;
    or_intrinsics K;
    R voxel, inv_voxel, tau, inv_tau, step_scale, block_metric;
    int pool, n_used, frame;
    /* open-addressing key -> block id (host structure; any exact map works) */
    unsigned long long *keys;
    int *ids;
    size_t hcap;
    int *bcoord; /* 3 per block */
    int *stamp;
#if OR_F64
    double *sdf, *w;
#else
    uint16_t *sdf; /* int16 bits (REF) or fp16 bits (HALF) */
    float *wf;     /* REF weight */
    uint16_t *w16; /* HALF weight */
#endif
    uint8_t *rgb; /* 4 per voxel */
    int *vis;
    int nvis;
    float *zr_min, *zr_max;
    int zr_w, zr_h, nrender;
};

typedef struct SFX(or_map) MAP;

static unsigned long long key_of(int x, int y, int z) {
    const unsigned long long m = (1ull << 21) - 1ull;
    return (((unsigned long long)(unsigned)x & m) << 42) | (((unsigned long long)(unsigned)y & m) << 21) |
           ((unsigned long long)(unsigned)z & m);
}
static size_t hslot(unsigned long long k, size_t cap) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33;
    return (size_t)(k & (cap - 1));
}
static int map_find(const MAP *m, int x, int y, int z) {
    const unsigned long long k = key_of(x, y, z);
    for (size_t s = hslot(k, m->hcap);; s = (s + 1) & (m->hcap - 1)) {
        if (m->keys[s] == ~0ull) return -1;
        if (m->keys[s] == k) return m->ids[s];
    }
}
/* createBlock (map_struct.cu:280-325) without the lossy try-once lock: a
 * sequential insert that never drops a block while the pool has room. */
static int map_insert(MAP *m, int x, int y, int z) {
    const unsigned long long k = key_of(x, y, z);
    size_t s = hslot(k, m->hcap);
    for (;; s = (s + 1) & (m->hcap - 1)) {
        if (m->keys[s] == k) return m->ids[s];
        if (m->keys[s] == ~0ull) break;
    }
    if (m->n_used >= m->pool) return -1;
    const int id = m->n_used++;
    m->keys[s] = k;
    m->ids[s] = id;
    m->bcoord[id * 3] = x; m->bcoord[id * 3 + 1] = y; m->bcoord[id * 3 + 2] = z;
    /* lazily zeroed block, as the product does at first integration */
    for (int i = 0; i < 512; ++i) {
        const size_t v = (size_t)id * 512 + i;
#if OR_F64
        m->sdf[v] = 0; m->w[v] = 0;
#else
        m->sdf[v] = 0;
        if (m->wf) m->wf[v] = 0;
        if (m->w16) m->w16[v] = 0;
#endif
        m->rgb[v * 4] = m->rgb[v * 4 + 1] = m->rgb[v * 4 + 2] = m->rgb[v * 4 + 3] = 0;
    }
    return id;
}

/* voxel storage semantics: Voxel::getSDF / setSDF / setWeight (voxel.h:36-66) */
static inline R vox_sdf(const MAP *m, size_t v) {
#if OR_F64
    return m->sdf[v];
#else
    if (m->cfg.voxel_layout == 0) return (float)(int16_t)m->sdf[v] / 32767.f;
    if (m->cfg.voxel_layout == 2) return (float)(int16_t)m->sdf[v] * 0x1.000202p-15f; /* 1/32767 rounded up */
    _Float16 h;
    memcpy(&h, &m->sdf[v], 2);
    return (float)h;
#endif
}
static inline R vox_w(const MAP *m, size_t v) {
#if OR_F64
    return m->w[v];
#else
    if (m->cfg.voxel_layout == 0) return m->wf[v];
    _Float16 h;
    memcpy(&h, &m->w16[v], 2);
    return (float)h;
#endif
}
static inline void vox_store(MAP *m, size_t v, R sdf, R w) {
#if OR_F64
    m->sdf[v] = sdf;
    m->w[v] = w > 255 ? 255 : w;
#else
    if (m->cfg.voxel_layout == 0) {
        m->sdf[v] = (uint16_t)(int16_t)or_trunc_sat(sdf * 32767.f);
        m->wf[v] = w > 255.f ? 255.f : w;
    } else {
        if (m->cfg.voxel_layout == 2) {
            m->sdf[v] = (uint16_t)(int16_t)or_trunc_sat(rint((double)(sdf * 32767.f))); /* __float2int_rn */
        } else {
            _Float16 h = (_Float16)sdf;
            memcpy(&m->sdf[v], &h, 2);
        }
        _Float16 hw = (_Float16)(w > 255.f ? 255.f : w);
        memcpy(&m->w16[v], &hw, 2);
    }
#endif
}

MAP *SFX(or_map_create)(const or_config *cfg, const or_intrinsics *K) {
    MAP *m = (MAP *)calloc(1, sizeof(MAP));
    if (!m) return NULL;
    m->cfg = *cfg;
    m->K = *K;
    m->voxel = TO_R(cfg->voxel_size);
    m->inv_voxel = (R)1 / m->voxel;
    m->tau = TO_R(cfg->truncation);
    m->inv_tau = INV_D(m->tau);
    m->step_scale = m->tau * m->inv_voxel;
    m->block_metric = (R)8 * m->voxel;
    m->pool = cfg->num_blocks;
    m->hcap = 64;
    while (m->hcap < (size_t)m->pool * 2) m->hcap <<= 1;
    m->keys = (unsigned long long *)malloc(m->hcap * sizeof(unsigned long long));
    m->ids = (int *)malloc(m->hcap * sizeof(int));
    memset(m->keys, 0xff, m->hcap * sizeof(unsigned long long));
    m->bcoord = (int *)malloc((size_t)m->pool * 3 * sizeof(int));
    m->stamp = (int *)calloc((size_t)m->pool, sizeof(int));
    const size_t nv = (size_t)m->pool * 512;
#if OR_F64
    m->sdf = (double *)malloc(nv * sizeof(double));
    m->w = (double *)malloc(nv * sizeof(double));
#else
    m->sdf = (uint16_t *)malloc(nv * 2);
    if (cfg->voxel_layout == 0) m->wf = (float *)malloc(nv * 4);
    else m->w16 = (uint16_t *)malloc(nv * 2);
#endif
    m->rgb = (uint8_t *)malloc(nv * 4);
    m->vis = (int *)malloc((size_t)m->pool * sizeof(int));
    m->zr_w = K->width / 8;
    m->zr_h = K->height / 8;
    m->zr_min = (float *)malloc((size_t)m->zr_w * m->zr_h * sizeof(float));
    m->zr_max = (float *)malloc((size_t)m->zr_w * m->zr_h * sizeof(float));
    return m;
}

void SFX(or_map_destroy)(MAP *m) {
    if (!m) return;
    free(m->keys); free(m->ids); free(m->bcoord); free(m->stamp); free(m->sdf);
#if !OR_F64
    free(m->wf); free(m->w16);
#else
    free(m->w);
#endif
    free(m->rgb); free(m->vis); free(m->zr_min); free(m->zr_max);
    free(m);
}

/* create_blocks_kernel (src/voxel_hashing/depth_fusion.cu:121-228): the blocks
 * of one pixel's truncation band, 3-D Bresenham between block_near / block_far */
static int pixel_blocks(const MAP *m, const M34 *T, int x, int y, R z, int *out /* 3*n */, int cap) {
    const or_intrinsics *K = &m->K;
    const R zmin = TO_R(m->cfg.zmin_update), zmax = TO_R(m->cfg.zmax_update);
    if (z != z || z < zmin || z > zmax) return 0;
    const R z_thresh = m->tau * (R)0.5;
    const R z_near = RFMAX(zmin, z - z_thresh), z_far = RFMIN(zmax, z + z_thresh);
    if (z_near >= z_far) return 0;
    const R invfx = (R)1 / TO_R(K->fx), invfy = (R)1 / TO_R(K->fy);
    int b[2][3];
    for (int s = 0; s < 2; ++s) {
        const R zz = s ? z_far : z_near;
        /* unproject (depth_fusion.cu:101-105): invfx * (x - cx) * z */
        const R px = (invfx * ((R)x - TO_R(K->cx))) * zz, py = (invfy * ((R)y - TO_R(K->cy))) * zz;
        const V3 w = m_apply(T, px, py, zz);
        b[s][0] = vtob(floor_r(w.x / m->voxel));
        b[s][1] = vtob(floor_r(w.y / m->voxel));
        b[s][2] = vtob(floor_r(w.z / m->voxel));
    }
    int n = 0;
    int bn[3] = {b[0][0], b[0][1], b[0][2]};
    const int d[3] = {b[1][0] - bn[0], b[1][1] - bn[1], b[1][2] - bn[2]};
    const int inc[3] = {d[0] < 0 ? -1 : 1, d[1] < 0 ? -1 : 1, d[2] < 0 ? -1 : 1};
    const int ab[3] = {abs(d[0]), abs(d[1]), abs(d[2])};
    const int e2[3] = {ab[0] << 1, ab[1] << 1, ab[2] << 1};
#define EMIT()                                                   \
    do {                                                         \
        if (n < cap) { out[3 * n] = bn[0]; out[3 * n + 1] = bn[1]; out[3 * n + 2] = bn[2]; } \
        ++n;                                                     \
    } while (0)
    EMIT();
    int major, a1, a2; /* the reference's err_1 / err_2 axes per branch */
    if (ab[0] >= ab[1] && ab[0] >= ab[2]) { major = 0; a1 = 1; a2 = 2; }
    else if (ab[1] >= ab[0] && ab[1] >= ab[2]) { major = 1; a1 = 0; a2 = 2; }
    else { major = 2; a1 = 1; a2 = 0; }
    int err1 = e2[a1] - 1, err2 = e2[a2] - 1;
    for (int i = 0; i < ab[major]; ++i) {
        if (err1 > 0) { bn[a1] += inc[a1]; err1 -= e2[major]; }
        if (err2 > 0) { bn[a2] += inc[a2]; err2 -= e2[major]; }
        err1 += e2[a1]; err2 += e2[a2];
        bn[major] += inc[major];
        EMIT();
    }
#undef EMIT
    return n;
}

/* is_block_visible (depth_fusion.cu:15-47) */
static int block_in_frustum(const MAP *m, const M34 *Tcw, const int *b) {
    const or_intrinsics *K = &m->K;
    for (int c = 0; c < 8; ++c) {
        const int cx = b[0] + ((c & 1) ? 1 : 0), cy = b[1] + ((c & 2) ? 1 : 0), cz = b[2] + ((c & 4) ? 1 : 0);
        const V3 p = m_apply(Tcw, (R)cx * m->block_metric, (R)cy * m->block_metric, (R)cz * m->block_metric);
        const R u = (TO_R(K->fx) * p.x) / p.z + TO_R(K->cx);
        const R v = (TO_R(K->fy) * p.y) / p.z + TO_R(K->cy);
        if (!(u < 0 || v < 0 || u > (R)(K->width - 1) || v > (R)(K->height - 1) || p.z < TO_R(m->cfg.zmin_update) ||
              p.z > TO_R(m->cfg.zmax_update)))
            return 1;
    }
    return 0;
}

/* update_map_with_colour_kernel (depth_fusion.cu:288-354) when nmap == NULL,
 * update_map_weighted_kernel (depth_fusion.cu:356-428) otherwise */
static void integrate_block(MAP *m, int id, const M34 *Tcw, const float *depth, const uint8_t *rgb, const float *nmap) {
    const or_intrinsics *K = &m->K;
    const int W = K->width, H = K->height;
    const int *bc = m->bcoord + id * 3;
    const R zmin = TO_R(m->cfg.zmin_update), zmax = TO_R(m->cfg.zmax_update);
    for (int li = 0; li < 512; ++li) {
        const int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
        const size_t vi = (size_t)id * 512 + li;
        const V3 p = m_apply(Tcw, (R)(bc[0] * 8 + lx) * m->voxel, (R)(bc[1] * 8 + ly) * m->voxel,
                             (R)(bc[2] * 8 + lz) * m->voxel);
        const int u = floor_rd(((TO_R(K->fx) * p.x) / p.z + TO_R(K->cx)) + (R)0.5);
        const int v = floor_rd(((TO_R(K->fy) * p.y) / p.z + TO_R(K->cy)) + (R)0.5);
        if (u < 0 || v < 0 || u > W - 1 || v > H - 1) continue;
        const R dist = TO_R(depth[(size_t)v * W + u]);
        R nz = 0;
        if (!nmap) {
            if (dist != dist || (double)dist < 1e-2 || dist > zmax || dist < zmin) continue;
        } else {
            const float *n = nmap + ((size_t)v * W + u) * 4;
            nz = TO_R(n[2]);
            if (dist != dist || n[0] != n[0] || dist > zmax || dist < zmin) continue;
        }
        R sdf = dist - p.z;
        if (sdf < -m->tau) continue;
        sdf = RFMIN((R)1, sdf * m->inv_tau);
        const R sdf_p = vox_sdf(m, vi), w_p = vox_w(m, vi);
        const R weight = !nmap ? (R)1 / (dist * dist) : RFABS(RSIN(nz)) / (dist * dist);
        const uint8_t *cn = rgb + ((size_t)v * W + u) * 3;
        uint8_t *cp = m->rgb + vi * 4;
        if (w_p == 0) {
            vox_store(m, vi, sdf, weight);
            cp[0] = cn[0]; cp[1] = cn[1]; cp[2] = cn[2];
            continue;
        }
        const R ns = (sdf_p * w_p + sdf * weight) / (w_p + weight);
        vox_store(m, vi, ns, w_p + weight);
        const R den = w_p + weight;
        for (int c = 0; c < 3; ++c) cp[c] = (uint8_t)or_trunc_sat(((R)cp[c] * w_p + (R)cn[c] * weight) / den);
    }
}

/* DenseMapping::update -> cuda::update / update_weighted (depth_fusion.cu:430-575) */
int SFX(or_fuse)(MAP *m, const float *depth, const uint8_t *rgb, const float *nmap, const double T[16]) {
    set_threads(m->cfg.threads);
    m->frame += 1;
    const or_intrinsics *K = &m->K;
    const int W = K->width, H = K->height;
    const M34 Twc = to_m(T);
    /* allocation: walks in parallel per row, inserts in pixel order */
    int **rows = (int **)calloc((size_t)H, sizeof(int *));
    int *rown = (int *)calloc((size_t)H, sizeof(int));
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; ++y) {
        int cap = 3 * 4 * W, n = 0;
        int *tmp = (int *)malloc((size_t)cap * sizeof(int));
        for (int x = 0; x < W; ++x) {
            int blk[3 * 64];
            int k = pixel_blocks(m, &Twc, x, y, TO_R(depth[(size_t)y * W + x]), blk, 64);
            if (k > 64) k = 64;
            if (3 * (n + k) > cap) {
                cap = 2 * cap + 3 * k;
                tmp = (int *)realloc(tmp, (size_t)cap * sizeof(int));
            }
            memcpy(tmp + 3 * n, blk, (size_t)k * 3 * sizeof(int));
            n += k;
        }
        rows[y] = tmp;
        rown[y] = n;
    }
    for (int y = 0; y < H; ++y) {
        for (int i = 0; i < rown[y]; ++i) {
            const int *b = rows[y] + 3 * i;
            const int id = map_insert(m, b[0], b[1], b[2]);
            if (id >= 0) m->stamp[id] = m->frame;
        }
        free(rows[y]);
    }
    free(rows);
    free(rown);

    /* visible = touched this fuse or in the frustum (check_visibility_flag_kernel,
     * depth_fusion.cu:49-83, without the stale-flag / wrong-slot effects) */
    double inv[12];
    pose_inv(T, inv);
    const M34 Tcw = to_m(inv);
    m->nvis = 0;
    char *v = (char *)malloc((size_t)m->n_used + 1);
#pragma omp parallel for schedule(static)
    for (int id = 0; id < m->n_used; ++id)
        v[id] = (m->stamp[id] == m->frame) || block_in_frustum(m, &Tcw, m->bcoord + id * 3);
    for (int id = 0; id < m->n_used; ++id)
        if (v[id]) m->vis[m->nvis++] = id;
    free(v);
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < m->nvis; ++i) integrate_block(m, m->vis[i], &Tcw, depth, rgb, nmap);
    return m->nvis;
}

/* ------------------------------------------------------------------ raycast */

/* create_rendering_block (ray_tracing.cu:63-126) + fill (:187-210); the union of
 * the 16x16 tiles of a block is its clamped box, so the box is filled directly */
static void zrange_pass(MAP *m, const M34 *Tcw) {
    const or_intrinsics *K = &m->K;
    const int n = m->zr_w * m->zr_h;
    for (int i = 0; i < n; ++i) { m->zr_min[i] = 100.f; m->zr_max[i] = 0.f; }
    m->nrender = 0;
    const R zmin_r = TO_R(m->cfg.zmin_raycast), zmax_r = TO_R(m->cfg.zmax_raycast);
    for (int b = 0; b < m->nvis; ++b) {
        const int *bc = m->bcoord + m->vis[b] * 3;
        int ulx = m->zr_w, uly = m->zr_h, lrx = -1, lry = -1;
        R zx = zmax_r, zy = zmin_r;
        for (int c = 0; c < 8; ++c) {
            const int cx = bc[0] + ((c & 1) ? 1 : 0), cy = bc[1] + ((c & 2) ? 1 : 0), cz = bc[2] + ((c & 4) ? 1 : 0);
            const V3 p = m_apply(Tcw, (R)cx * m->block_metric, (R)cy * m->block_metric, (R)cz * m->block_metric);
            const R u = ((TO_R(K->fx) * p.x) / p.z + TO_R(K->cx)) / (R)8;
            const R v = ((TO_R(K->fy) * p.y) / p.z + TO_R(K->cy)) / (R)8;
            const R fu = RFLOOR(u), fv = RFLOOR(v), cu = RCEIL(u), cv = RCEIL(v);
            if ((R)ulx > fu) ulx = or_trunc_sat(fu);
            if ((R)lrx < cu) lrx = or_trunc_sat(cu);
            if ((R)uly > fv) uly = or_trunc_sat(fv);
            if ((R)lry < cv) lry = or_trunc_sat(cv);
            if (zx > p.z) zx = p.z;
            if (zy < p.z) zy = p.z;
        }
        if (ulx < 0) ulx = 0;
        if (uly < 0) uly = 0;
        if (lrx >= m->zr_w) lrx = m->zr_w - 1;
        if (lry >= m->zr_h) lry = m->zr_h - 1;
        if (ulx > lrx || uly > lry) continue;
        if (zx < zmin_r) zx = zmin_r;
        if (zy < zmin_r) continue;
        m->nrender++;
        for (int y = uly; y <= lry; ++y)
            for (int x = ulx; x <= lrx; ++x) {
                float *a = &m->zr_min[y * m->zr_w + x], *bb = &m->zr_max[y * m->zr_w + x];
                if ((float)zx < *a) *a = (float)zx;
                if ((float)zy > *bb) *bb = (float)zy;
            }
    }
}

/* march statistics for the raycast roofline: samples, trilinear reads, steps, rays */
typedef struct { long long samples, interps, steps, rays, hits, empty, missing; } RayStats;
static _Thread_local RayStats *g_rs;

/* read_sdf (ray_tracing.cu:291-305) */
static R read_sdf(const MAP *m, R px, R py, R pz, int *valid) {
    if (g_rs) g_rs->samples++;
    const int vx = floor_r(px), vy = floor_r(py), vz = floor_r(pz);
    const int id = map_find(m, vtob(vx), vtob(vy), vtob(vz));
    if (id < 0 && g_rs) g_rs->missing++;
    if (id >= 0) {
        const size_t i = (size_t)id * 512 + vtol(vz) * 64 + vtol(vy) * 8 + vtol(vx);
        if (vox_w(m, i) != 0) {
            *valid = 1;
            return vox_sdf(m, i);
        }
    }
    *valid = 0;
    return (R)NAN;
}

/* read_sdf_interped (ray_tracing.cu:307-339) */
static R read_interp(const MAP *m, R px, R py, R pz, int *valid) {
    if (g_rs) g_rs->interps++;
    const R fx = px - RFLOOR(px), fy = py - RFLOOR(py), fz = pz - RFLOOR(pz);
    int vp, v;
    R s0, s1, r0, r1, r2, r3;
    s0 = read_sdf(m, px, py, pz, &vp);
    s1 = read_sdf(m, px + (R)1, py + (R)0, pz + (R)0, &v); vp &= v;
    r0 = ((R)1 - fx) * s0 + fx * s1;
    s0 = read_sdf(m, px + (R)0, py + (R)1, pz + (R)0, &v); vp &= v;
    s1 = read_sdf(m, px + (R)1, py + (R)1, pz + (R)0, &v); vp &= v;
    r1 = ((R)1 - fx) * s0 + fx * s1;
    r2 = ((R)1 - fy) * r0 + fy * r1;
    s0 = read_sdf(m, px + (R)0, py + (R)0, pz + (R)1, &v); vp &= v;
    s1 = read_sdf(m, px + (R)1, py + (R)0, pz + (R)1, &v); vp &= v;
    r0 = ((R)1 - fx) * s0 + fx * s1;
    s0 = read_sdf(m, px + (R)0, py + (R)1, pz + (R)1, &v); vp &= v;
    s1 = read_sdf(m, px + (R)1, py + (R)1, pz + (R)1, &v); vp &= v;
    r1 = ((R)1 - fx) * s0 + fx * s1;
    r3 = ((R)1 - fy) * r0 + fy * r1;
    *valid = vp;
    return ((R)1 - fz) * r2 + fz * r3;
}

/* MapRenderingDelegate::operator() (ray_tracing.cu:346-425) */
/* read_colour (ray_tracing.cu:427-441): the colour of the voxel ToVector3i(pt),
 * valid when its weight is not 0 */
static int read_colour(const MAP *m, R px, R py, R pz, uint8_t *rgb) {
    const int vx = floor_r(px), vy = floor_r(py), vz = floor_r(pz);
    const int id = map_find(m, vtob(vx), vtob(vy), vtob(vz));
    if (id < 0) return 0;
    const size_t i = (size_t)id * 512 + vtol(vz) * 64 + vtol(vy) * 8 + vtol(vx);
    if (vox_w(m, i) == 0) return 0;
    rgb[0] = m->rgb[i * 4]; rgb[1] = m->rgb[i * 4 + 1]; rgb[2] = m->rgb[i * 4 + 2];
    return 1;
}

/* rgb (optional, 3 bytes): the colour raycast_with_colour (ray_tracing.cu:478-564)
 * means to write -- the hit's nearest voxel colour, white (255) elsewhere; the
 * vertex keeps the march's own validity, as the executed raycast does */
static void ray_pixel(const MAP *m, const M34 *Twc, const M34 *Tcw, int x, int y, float *out, uint8_t *rgb) {
    const or_intrinsics *K = &m->K;
    out[0] = out[1] = out[2] = out[3] = NAN;
    if (rgb) rgb[0] = rgb[1] = rgb[2] = 255;
    const int cx = floor_rd((R)x / (R)8), cy = floor_rd((R)y / (R)8);
    if (cx >= m->zr_w || cy >= m->zr_h) return;
    const R zr0 = m->zr_min[cy * m->zr_w + cx], zr1 = m->zr_max[cy * m->zr_w + cx];
    if ((double)zr1 < 1e-3 || (double)zr0 < 1e-3 || zr0 != zr0 || zr1 != zr1) return;
    const R invfx = (R)1 / TO_R(K->fx), invfy = (R)1 / TO_R(K->fy);
    const R iv = m->inv_voxel;
    R ux = (((R)x - TO_R(K->cx)) * invfx) * zr0, uy = (((R)y - TO_R(K->cy)) * invfy) * zr0;
    R dist_s = n3(ux, uy, zr0) * iv;
    V3 bs = m_apply(Twc, ux, uy, zr0);
    bs = v3(bs.x * iv, bs.y * iv, bs.z * iv);
    ux = (((R)x - TO_R(K->cx)) * invfx) * zr1;
    uy = (((R)y - TO_R(K->cy)) * invfy) * zr1;
    const R dist_e = n3(ux, uy, zr1) * iv;
    V3 be = m_apply(Twc, ux, uy, zr1);
    be = v3(be.x * iv, be.y * iv, be.z * iv);
    V3 dir = v3(be.x - bs.x, be.y - bs.y, be.z - bs.z);
    const R dn = n3(dir.x, dir.y, dir.z);
    dir = v3(dir.x / dn, dir.y / dn, dir.z / dn);
    V3 r = bs;
    R sdf = 1, last_sdf, step;
    int valid = 0;
    if (g_rs) g_rs->rays++;
    for (int it = 0; dist_s < dist_e && it < (1 << 16); ++it) {
        if (g_rs) g_rs->steps++;
        last_sdf = sdf;
        sdf = read_sdf(m, r.x, r.y, r.z, &valid);
        if (sdf <= (R)0.5 && sdf >= (R)-0.5) sdf = read_interp(m, r.x, r.y, r.z, &valid);
        if (sdf <= 0) break;
        if (sdf >= 0 && last_sdf < 0) return;
        step = valid ? RFMAX(sdf * m->step_scale, (R)1) : (R)2;
        if (g_rs && !valid) g_rs->empty++;
        r = v3(r.x + dir.x * step, r.y + dir.y * step, r.z + dir.z * step);
        dist_s += step;
    }
    int found = 0;
    if (sdf <= 0) {
        step = sdf * m->step_scale;
        r = v3(r.x + dir.x * step, r.y + dir.y * step, r.z + dir.z * step);
        sdf = read_interp(m, r.x, r.y, r.z, &valid);
        step = sdf * m->step_scale;
        r = v3(r.x + dir.x * step, r.y + dir.y * step, r.z + dir.z * step);
        found = valid;
    }
    if (found) {
        if (g_rs) g_rs->hits++;
        const V3 c = m_apply(Tcw, r.x * m->voxel, r.y * m->voxel, r.z * m->voxel);
        out[0] = (float)c.x; out[1] = (float)c.y; out[2] = (float)c.z; out[3] = 1.0f;
        uint8_t col[3];
        if (rgb && read_colour(m, r.x, r.y, r.z, col)) { rgb[0] = col[0]; rgb[1] = col[1]; rgb[2] = col[2]; }
    }
}

int SFX(or_raycast_maps)(MAP *m, const double T[16], float *vmap, uint8_t *rgb) {
    set_threads(m->cfg.threads);
    double inv[12];
    pose_inv(T, inv);
    const M34 Twc = to_m(T), Tcw = to_m(inv);
    zrange_pass(m, &Tcw);
    /* DenseMapping::raycast returns early without visible or renderable blocks
     * (voxel_hashing.cpp:92-93, 105) and leaves vmap untouched */
    if (m->nvis == 0 || m->nrender == 0) return 0;
    const int W = m->K.width, H = m->K.height;
#pragma omp parallel for schedule(dynamic, 2)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            ray_pixel(m, &Twc, &Tcw, x, y, vmap + ((size_t)y * W + x) * 4, rgb ? rgb + ((size_t)y * W + x) * 3 : NULL);
    return 1;
}

int SFX(or_raycast)(MAP *m, const double T[16], float *vmap) { return SFX(or_raycast_maps)(m, T, vmap, NULL); }

/* DenseMapping::raycast_check_visibility (voxel_hashing.cpp:121-135): the visible
 * list recomputed for pose T by count_visible_entry (ray_tracing.cu:778-807) --
 * every allocated block with a corner in the frustum (is_block_visible), no
 * "touched" term -- then raycast at T.  The reference's functor also tests empty
 * entries and reads an uninitialised entry count (ray_tracing.cu:726-743); only
 * allocated blocks are taken here. */
int SFX(or_raycast_check_visibility)(MAP *m, const double T[16], float *vmap) {
    set_threads(m->cfg.threads);
    double inv[12];
    pose_inv(T, inv);
    const M34 Tcw = to_m(inv);
    char *v = (char *)malloc((size_t)m->n_used + 1);
#pragma omp parallel for schedule(static)
    for (int id = 0; id < m->n_used; ++id) v[id] = block_in_frustum(m, &Tcw, m->bcoord + id * 3);
    m->nvis = 0;
    for (int id = 0; id < m->n_used; ++id)
        if (v[id]) m->vis[m->nvis++] = id;
    free(v);
    return SFX(or_raycast)(m, T, vmap);
}

/* counts of the last fuse's raycast at pose T (single thread): rays marched,
 * march steps, voxel samples (each a hash lookup + one voxel read), trilinear
 * reads, hits */
void SFX(or_ray_stats)(MAP *m, const double T[16], long long out[7], int32_t *steps_per_pixel) {
    double inv[12];
    pose_inv(T, inv);
    const M34 Twc = to_m(T), Tcw = to_m(inv);
    zrange_pass(m, &Tcw);
    RayStats rs = {0, 0, 0, 0, 0, 0, 0};
    g_rs = &rs;
    float px[4];
    if (m->nvis && m->nrender)
        for (int y = 0; y < m->K.height; ++y)
            for (int x = 0; x < m->K.width; ++x) {
                const long long s0 = rs.steps + rs.interps * 8;
                ray_pixel(m, &Twc, &Tcw, x, y, px, NULL);
                if (steps_per_pixel) steps_per_pixel[y * m->K.width + x] = (int32_t)(rs.steps + rs.interps * 8 - s0);
            }
    g_rs = NULL;
    out[0] = rs.rays; out[1] = rs.steps; out[2] = rs.samples; out[3] = rs.interps; out[4] = rs.hits;
    out[5] = rs.empty; out[6] = rs.missing;
}

int64_t SFX(or_map_blocks)(const MAP *m) { return m->n_used; }

int64_t SFX(or_map_export)(const MAP *m, int32_t *coords, float *sdf, float *w, uint8_t *rgb, int64_t max_blocks) {
    const int64_t n = m->n_used < max_blocks ? m->n_used : max_blocks;
    for (int64_t b = 0; b < n; ++b) {
        for (int k = 0; k < 3; ++k) coords[b * 3 + k] = m->bcoord[b * 3 + k];
        for (int i = 0; i < 512; ++i) {
            const size_t v = (size_t)b * 512 + i;
            sdf[v] = (float)vox_sdf(m, v);
            w[v] = (float)vox_w(m, v);
            for (int c = 0; c < 3; ++c) rgb[v * 3 + c] = m->rgb[v * 4 + c];
        }
    }
    return n;
}

int64_t SFX(or_visible)(const MAP *m, int32_t *coords, int64_t max_blocks) {
    const int64_t n = m->nvis < max_blocks ? m->nvis : max_blocks;
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) coords[i * 3 + k] = m->bcoord[m->vis[i] * 3 + k];
    return m->nvis;
}

void SFX(or_zrange)(const MAP *m, float *out) {
    for (int i = 0; i < m->zr_w * m->zr_h; ++i) {
        out[2 * i] = m->zr_min[i];
        out[2 * i + 1] = m->zr_max[i];
    }
}

int32_t SFX(or_render_blocks)(const MAP *m) { return m->nrender; }

/* ------------------------------------------------------------ marching cubes */

/* BuildVertexArray / BuildVertexAndColourArray (scene_mesh.cu:54-247, 393-588),
 * emitting blocks in id order, voxels in index order, triangles in table order */
int64_t SFX(or_mesh)(const MAP *m, int mode, float *vtx, void *attr, int64_t max_tris) {
    static const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    static const int edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                    {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    int64_t nt = 0;
    for (int b = 0; b < m->n_used; ++b) {
        const int *bc = m->bcoord + b * 3;
        for (int li = 0; li < 512; ++li) {
            const int pos[3] = {bc[0] * 8 + (li & 7), bc[1] * 8 + ((li >> 3) & 7), bc[2] * 8 + (li >> 6)};
            R s[8];
            uint8_t col[8][3];
            int ok = 1;
            for (int k = 0; k < 8 && ok; ++k) {
                const int v[3] = {pos[0] + corner[k][0], pos[1] + corner[k][1], pos[2] + corner[k][2]};
                const int id = map_find(m, vtob(v[0]), vtob(v[1]), vtob(v[2]));
                if (id < 0) { ok = 0; break; }
                const size_t vi = (size_t)id * 512 + vtol(v[2]) * 64 + vtol(v[1]) * 8 + vtol(v[0]);
                const R w = vox_w(m, vi);
                if (mode == 2 ? !((double)w > 1e-3) : (w == 0)) { ok = 0; break; }
                s[k] = vox_sdf(m, vi);
                for (int c = 0; c < 3; ++c) col[k][c] = m->rgb[vi * 4 + c];
            }
            if (!ok) continue;
            int ci = 0;
            for (int k = 0; k < 8; ++k)
                if (s[k] < 0) ci |= 1 << k;
            const int em = or_edge_table(ci);
            if (ci <= 0 || em == 0) continue;
            R ev[12][3];
            for (int e = 0; e < 12; ++e) {
                if (!((em >> e) & 1)) continue;
                const R v1 = s[edge[e][0]], v2 = s[edge[e][1]];
                R val;
                /* interpolate_sdf (scene_mesh.cu:108-117) */
                if ((double)RFABS(0 - v1) < 1e-6) val = 0;
                else if ((double)RFABS(0 - v2) < 1e-6) val = 1;
                else if ((double)RFABS(v1 - v2) < 1e-6) val = 0;
                else val = (0 - v1) / (v2 - v1);
                R o[3];
                switch (e) {
                    case 0: o[0] = val; o[1] = 0; o[2] = 0; break;
                    case 1: o[0] = 1; o[1] = val; o[2] = 0; break;
                    case 2: o[0] = 1 - val; o[1] = 1; o[2] = 0; break;
                    case 3: o[0] = 0; o[1] = 1 - val; o[2] = 0; break;
                    case 4: o[0] = val; o[1] = 0; o[2] = 1; break;
                    case 5: o[0] = 1; o[1] = val; o[2] = 1; break;
                    case 6: o[0] = 1 - val; o[1] = 1; o[2] = 1; break;
                    case 7: o[0] = 0; o[1] = 1 - val; o[2] = 1; break;
                    case 8: o[0] = 0; o[1] = 0; o[2] = val; break;
                    case 9: o[0] = 1; o[1] = 0; o[2] = val; break;
                    case 10: o[0] = 1; o[1] = 1; o[2] = val; break;
                    default: o[0] = 0; o[1] = 1; o[2] = val; break;
                }
                for (int k = 0; k < 3; ++k) ev[e][k] = ((R)pos[k] + o[k]) * m->voxel;
            }
            int tri[16];
            const int n = or_tri_table(ci, tri);
            for (int t = 0; t < n; t += 3, ++nt) {
                if (nt >= max_tris) continue;
                R *a = ev[tri[t]], *bb = ev[tri[t + 1]], *c = ev[tri[t + 2]];
                for (int k = 0; k < 3; ++k) {
                    vtx[nt * 9 + k] = (float)a[k];
                    vtx[nt * 9 + 3 + k] = (float)bb[k];
                    vtx[nt * 9 + 6 + k] = (float)c[k];
                }
                if (mode == 1 && attr) {
                    const V3 u = v3(bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]);
                    const V3 w = v3(c[0] - a[0], c[1] - a[1], c[2] - a[2]);
                    const V3 nn = cross(u, w);
                    const R l = n3(nn.x, nn.y, nn.z);
                    float *na = (float *)attr + nt * 9;
                    for (int q = 0; q < 3; ++q) {
                        na[q * 3] = (float)(nn.x / l); na[q * 3 + 1] = (float)(nn.y / l); na[q * 3 + 2] = (float)(nn.z / l);
                    }
                } else if (mode == 2 && attr) {
                    uint8_t *ca = (uint8_t *)attr + nt * 9;
                    for (int q = 0; q < 3; ++q) {
                        const int e = tri[t + q];
                        const int cr = e < 8 ? e : e - 8;
                        for (int k = 0; k < 3; ++k) ca[q * 3 + k] = col[cr][k];
                    }
                }
            }
        }
    }
    return nt;
}

/* ================================================================ pyramids */

struct SFX(or_frame) {
    or_config cfg;
    int levels;
    int w[OR_MAX_LEVELS], h[OR_MAX_LEVELS];
    R fx[OR_MAX_LEVELS], fy[OR_MAX_LEVELS], cx[OR_MAX_LEVELS], cy[OR_MAX_LEVELS], ifx[OR_MAX_LEVELS], ify[OR_MAX_LEVELS];
    R *depth[OR_MAX_LEVELS], *inten[OR_MAX_LEVELS], *gx[OR_MAX_LEVELS], *gy[OR_MAX_LEVELS];
    R *vmap[OR_MAX_LEVELS], *nmap[OR_MAX_LEVELS]; /* 4 per pixel */
};
typedef struct SFX(or_frame) FRAME;

FRAME *SFX(or_frame_create)(const or_config *cfg, const or_intrinsics *K) {
    FRAME *f = (FRAME *)calloc(1, sizeof(FRAME));
    f->cfg = *cfg;
    f->levels = cfg->num_levels;
    /* IntrinsicMatrix + pyr_down (include/data_struct/intrinsic_matrix.h:27-37) */
    float fx = K->fx, fy = K->fy, cx = K->cx, cy = K->cy;
    int w = K->width, h = K->height;
    for (int l = 0; l < f->levels; ++l) {
        f->w[l] = w; f->h[l] = h;
        f->fx[l] = TO_R(fx); f->fy[l] = TO_R(fy); f->cx[l] = TO_R(cx); f->cy[l] = TO_R(cy);
        f->ifx[l] = TO_R(1.0f / fx); f->ify[l] = TO_R(1.0f / fy);
        const size_t p = (size_t)w * h;
        f->depth[l] = (R *)calloc(p, sizeof(R));
        f->inten[l] = (R *)calloc(p, sizeof(R));
        f->gx[l] = (R *)calloc(p, sizeof(R));
        f->gy[l] = (R *)calloc(p, sizeof(R));
        f->vmap[l] = (R *)calloc(p * 4, sizeof(R));
        f->nmap[l] = (R *)calloc(p * 4, sizeof(R));
        w = (int)(0.5f * (float)w); h = (int)(0.5f * (float)h);
        fx = 0.5f * fx; fy = 0.5f * fy; cx = 0.5f * cx; cy = 0.5f * cy;
    }
    return f;
}

void SFX(or_frame_destroy)(FRAME *f) {
    if (!f) return;
    for (int l = 0; l < f->levels; ++l) {
        free(f->depth[l]); free(f->inten[l]); free(f->gx[l]); free(f->gy[l]); free(f->vmap[l]); free(f->nmap[l]);
    }
    free(f);
}

static inline int refl(int i, int n) {
    if (i < 0) i = -i;
    if (i >= n) i = 2 * n - 2 - i;
    return i;
}

/* backProjectDepthK (src/tracking/cuda_imgproc.cu:249-263) */
static inline void backproj(const FRAME *f, int l, int x, int y, R *o) {
    const R z = f->depth[l][(size_t)y * f->w[l] + x];
    if (z > (R)0.3f && z < (R)5.0f) {
        o[0] = (z * ((R)x - f->cx[l])) * f->ifx[l];
        o[1] = (z * ((R)y - f->cy[l])) * f->ify[l];
        o[2] = z;
        o[3] = 1;
    } else {
        o[0] = o[1] = o[2] = (R)NAN;
        o[3] = -1;
    }
}

/* computeNMapK (cuda_imgproc.cu:276-294) from the vertex map of level l */
static void nmap_level(FRAME *f, int l) {
    const int w = f->w[l], h = f->h[l];
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            R *n = f->nmap[l] + ((size_t)y * w + x) * 4;
            if (x < w - 1 && y < h - 1) {
                const int x10 = x > 0 ? x - 1 : 0, y10 = y > 0 ? y - 1 : 0;
                const R *v00 = f->vmap[l] + ((size_t)y * w + x10) * 4, *v01 = f->vmap[l] + ((size_t)y * w + x + 1) * 4;
                const R *v10 = f->vmap[l] + ((size_t)y10 * w + x) * 4, *v11 = f->vmap[l] + ((size_t)(y + 1) * w + x) * 4;
                const V3 a = v3(v01[0] - v00[0], v01[1] - v00[1], v01[2] - v00[2]);
                const V3 b = v3(v11[0] - v10[0], v11[1] - v10[1], v11[2] - v10[2]);
                const V3 c = cross(a, b);
                const R len = n3(c.x, c.y, c.z);
                n[0] = c.x / len; n[1] = c.y / len; n[2] = c.z / len; n[3] = 1;
            } else {
                n[0] = n[1] = n[2] = n[3] = (R)NAN; /* unwritten in the reference */
            }
        }
}

/* DeviceImage::upload (src/tracking/device_image.cpp:146-181) */
void SFX(or_build_pyramid)(FRAME *f, const float *depth, const uint8_t *rgb) {
    set_threads(f->cfg.threads);
    const int W = f->w[0], H = f->h[0];
    /* filterDepthBilateral (cuda_imgproc.cu:197-200): circular window radius 2,
     * sigma_space = sigma_colour = 1, reflect-101 border */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const R c = TO_R(depth[(size_t)y * W + x]);
            if (!f->cfg.bilateral) { f->depth[0][(size_t)y * W + x] = c; continue; }
            R s1 = 0, s2 = 0;
            for (int dy = -2; dy <= 2; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    const int sp = dx * dx + dy * dy;
                    if (sp > 4) continue;
                    const R v = TO_R(depth[(size_t)refl(y + dy, H) * W + refl(x + dx, W)]);
                    const R d = v - c;
                    const R w = REXP((R)sp * (R)-0.5 + (d * d) * (R)-0.5);
                    s1 += w * v;
                    s2 += w;
                }
            f->depth[0][(size_t)y * W + x] = s1 / s2;
        }
    /* cvtColor RGB2GRAY on float RGB (device_image.cpp:161-162) */
    for (size_t p = 0; p < (size_t)W * H; ++p)
        f->inten[0][p] = ((R)0.299f * (R)rgb[p * 3] + (R)0.587f * (R)rgb[p * 3 + 1]) + (R)0.114f * (R)rgb[p * 3 + 2];
    for (int l = 1; l < f->levels; ++l) {
        const int w = f->w[l], h = f->h[l], pw = f->w[l - 1], ph = f->h[l - 1];
        const R *sd = f->depth[l - 1], *si = f->inten[l - 1];
#pragma omp parallel for schedule(static)
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                /* cv::cuda::resize(0.5): 2x2 mean */
                const R a0 = sd[(size_t)(2 * y) * pw + 2 * x], a1 = sd[(size_t)(2 * y) * pw + 2 * x + 1];
                const R a2 = sd[(size_t)(2 * y + 1) * pw + 2 * x], a3 = sd[(size_t)(2 * y + 1) * pw + 2 * x + 1];
                f->depth[l][(size_t)y * w + x] = (((a0 + a1) + a2) + a3) * (R)0.25;
                /* cv::cuda::pyrDown: [1 4 6 4 1]/16 separable, reflect-101 */
                int xs[5];
                for (int k = 0; k < 5; ++k) xs[k] = refl(2 * x + k - 2, pw);
                R hr[5];
                for (int j = 0; j < 5; ++j) {
                    const R *row = si + (size_t)refl(2 * y + j - 2, ph) * pw;
                    hr[j] = (((row[xs[0]] + (R)4 * row[xs[1]]) + (R)6 * row[xs[2]]) + (R)4 * row[xs[3]]) + row[xs[4]];
                }
                f->inten[l][(size_t)y * w + x] =
                    ((((hr[0] + (R)4 * hr[1]) + (R)6 * hr[2]) + (R)4 * hr[3]) + hr[4]) * ((R)1 / (R)256);
            }
    }
    for (int l = 0; l < f->levels; ++l) {
        const int w = f->w[l], h = f->h[l];
        const R *I = f->inten[l];
#pragma omp parallel for schedule(static)
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const size_t p = (size_t)y * w + x;
                /* computeDerivativeK (cuda_imgproc.cu:217-234) */
                if (x < w - 1 && y < h - 1) {
                    const int x10 = x > 0 ? x - 1 : 0, y10 = y > 0 ? y - 1 : 0;
                    f->gx[l][p] = (I[(size_t)y * w + x + 1] - I[(size_t)y * w + x10]) * (R)0.5;
                    f->gy[l][p] = (I[(size_t)(y + 1) * w + x] - I[(size_t)y10 * w + x]) * (R)0.5;
                } else {
                    f->gx[l][p] = 0;
                    f->gy[l][p] = 0;
                }
                backproj(f, l, x, y, f->vmap[l] + p * 4);
            }
        nmap_level(f, l);
    }
}

void SFX(or_frame_get)(const FRAME *f, int kind, int level, float *out) {
    const size_t p = (size_t)f->w[level] * f->h[level];
    const R *src;
    size_t n = p;
    switch (kind) {
        case 0: src = f->vmap[level]; n = p * 4; break;
        case 1: src = f->nmap[level]; n = p * 4; break;
        case 2: src = f->inten[level]; break;
        case 3: src = f->gx[level]; break;
        case 4: src = f->gy[level]; break;
        default: src = f->depth[level]; break;
    }
    for (size_t i = 0; i < n; ++i) out[i] = (float)src[i];
}

/* after a raycast: level-0 vertex map replaced, finer levels by 2x2 mean,
 * normals recomputed (DeviceImage::resize_device_map, device_image.cpp:188-199) */
static void resize_device_map(FRAME *f) {
    for (int l = 1; l < f->levels; ++l) {
        const int w = f->w[l], h = f->h[l], pw = f->w[l - 1];
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const R *a = f->vmap[l - 1] + ((size_t)(2 * y) * pw + 2 * x) * 4, *b = a + 4;
                const R *c = f->vmap[l - 1] + ((size_t)(2 * y + 1) * pw + 2 * x) * 4, *d = c + 4;
                R *o = f->vmap[l] + ((size_t)y * w + x) * 4;
                for (int k = 0; k < 4; ++k) o[k] = (((a[k] + b[k]) + c[k]) + d[k]) * (R)0.25;
            }
    }
    for (int l = 0; l < f->levels; ++l) nmap_level(f, l);
}

void SFX(or_frame_set_vmap)(FRAME *f, const float *vmap0) {
    const size_t p = (size_t)f->w[0] * f->h[0];
    for (size_t i = 0; i < p * 4; ++i) f->vmap[0][i] = TO_R(vmap0[i]);
    resize_device_map(f);
}

/* ============================================================== reductions */

static inline R interp2(const R *img, int w, R x, R y) {
    const int u = (int)RFLOOR(x), v = (int)RFLOOR(y);
    const R ax = x - (R)u, ay = y - (R)v;
    const R *r0 = img + (size_t)v * w, *r1 = r0 + w;
    return (r0[u] * ((R)1 - ax) + r0[u + 1] * ax) * ((R)1 - ay) + (r1[u] * ((R)1 - ax) + r1[u + 1] * ax) * ay;
}

/* ICPReduction::searchPoint + getRow (src/tracking/pose_estimator.cu:168-222) */
static int icp_row(const FRAME *ref, const FRAME *cur, int l, const M34 *T, int p, R row[7]) {
    const R *vl = ref->vmap[l] + (size_t)p * 4;
    if (vl[0] != vl[0]) return 0;
    const V3 vg = m_apply(T, vl[0], vl[1], vl[2]);
    const R invz = INV_D(vg.z);
    const int u = floor_rd(((vg.x * invz) * cur->fx[l] + cur->cx[l]) + (R)0.5);
    const int v = floor_rd(((vg.y * invz) * cur->fy[l] + cur->cy[l]) + (R)0.5);
    const int w = cur->w[l], h = cur->h[l];
    if (u < 0 || v < 0 || u >= w || v >= h) return 0;
    const size_t q = (size_t)v * w + u;
    const R *vc = cur->vmap[l] + q * 4, *nl = ref->nmap[l] + (size_t)p * 4, *nc = cur->nmap[l] + q * 4;
    const V3 ng = m_rotate(T, nl[0], nl[1], nl[2]);
    const R dist = n3(vg.x - vc[0], vg.y - vc[1], vg.z - vc[2]);
    const V3 cr = cross(v3(nc[0], nc[1], nc[2]), ng);
    const R sine = n3(cr.x, cr.y, cr.z);
    if (!(sine < TO_R(ref->cfg.icp_angle_thresh) && dist <= TO_R(ref->cfg.icp_dist_thresh) && nc[0] == nc[0] &&
          ng.x == ng.x))
        return 0;
    const V3 vxn = cross(vg, ng);
    row[0] = ng.x; row[1] = ng.y; row[2] = ng.z;
    row[3] = vxn.x; row[4] = vxn.y; row[5] = vxn.z;
    row[6] = dot(ng, v3(vc[0] - vg.x, vc[1] - vg.y, vc[2] - vg.z));
    return 1;
}

/* RgbReduction2::find_corresp + compute_jacobian (src/tracking/m_estimator.cu:315-391) */
static int rgb_row(const FRAME *ref, const FRAME *cur, int l, const M34 *T, R stddev, int p, R row[7]) {
    const R *pt = ref->vmap[l] + (size_t)p * 4;
    if (pt[3] < 0 || pt[0] != pt[0]) return 0;
    const R il = ref->inten[l][p];
    if (!isfinite(il)) return 0;
    const V3 q = m_apply(T, pt[0], pt[1], pt[2]);
    const R u0 = (q.x / q.z) * cur->fx[l] + cur->cx[l];
    const R v0 = (q.y / q.z) * cur->fy[l] + cur->cy[l];
    const int w = cur->w[l], h = cur->h[l];
    if (!(u0 >= 2 && u0 < (R)(w - 2) && v0 >= 2 && v0 < (R)(h - 2))) return 0;
    const R ic = interp2(cur->inten[l], w, u0, v0);
    const R dx = interp2(cur->gx[l], w, u0, v0);
    const R dy = interp2(cur->gy[l], w, u0, v0);
    if (!((dx > 2 || dy > 2) && isfinite(ic) && isfinite(dx) && isfinite(dy))) return 0;
    const R zi = INV_D(q.z);
    const R lx = (dx * cur->fx[l]) * zi, ly = (dy * cur->fy[l]) * zi;
    const R lz = (-(lx * q.x + ly * q.y)) * zi;
    R res = ic - il;
    if ((double)stddev > 10e-5) res /= stddev;
    const R hub = HUBER_TH(stddev);
    R wgt = 1;
    if (RFABS(res) > hub && (double)stddev > 10e-6) wgt = RSQRT(hub / RFABS(res));
    const V3 pl = cross(q, v3(lx, ly, lz));
    row[0] = lx * wgt; row[1] = ly * wgt; row[2] = lz * wgt;
    row[3] = pl.x * wgt; row[4] = pl.y * wgt; row[5] = pl.z * wgt;
    row[6] = wgt * (-res);
    return 1;
}

/* sums in FP64 per row of pixels, rows combined in order (thread-count independent) */
void SFX(or_reduce)(const FRAME *ref, const FRAME *cur, int l, const float Tf[12], float stddev, double out[58]) {
    set_threads(ref->cfg.threads);
    M34 T;
    for (int i = 0; i < 12; ++i) T.m[i] = TO_R(Tf[i]);
    const int w = ref->w[l], h = ref->h[l];
    double *rows = (double *)calloc((size_t)h * 58, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        double *acc = rows + (size_t)y * 58;
        for (int x = 0; x < w; ++x) {
            const int p = y * w + x;
            R row[7];
            for (int part = 0; part < 2; ++part) {
                const int ok = part == 0 ? icp_row(ref, cur, l, &T, p, row) : rgb_row(ref, cur, l, &T, TO_R(stddev), p, row);
                if (!ok) continue;
                double *a = acc + 29 * part;
                int k = 0;
                for (int i = 0; i < 7; ++i)
                    for (int j = i; j < 7; ++j) a[k++] += (double)(row[i] * row[j]);
                a[28] += 1.0;
            }
        }
    }
    for (int k = 0; k < 58; ++k) out[k] = 0;
    for (int y = 0; y < h; ++y)
        for (int k = 0; k < 58; ++k) out[k] += rows[(size_t)y * 58 + k];
    free(rows);
}

/* The terms or_reduce adds, per pixel: the 28 products of each row's upper
 * triangle rounded to float, and 1 for the count (reduce_sum.h:48-61). */
void SFX(or_reduce_terms)(const FRAME *ref, const FRAME *cur, int l, const float Tf[12], float stddev, float *terms) {
    set_threads(ref->cfg.threads);
    M34 T;
    for (int i = 0; i < 12; ++i) T.m[i] = TO_R(Tf[i]);
    const int n = ref->w[l] * ref->h[l];
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n; ++p) {
        float *t = terms + (size_t)p * 58;
        for (int k = 0; k < 58; ++k) t[k] = 0.f;
        R row[7];
        for (int part = 0; part < 2; ++part) {
            const int ok = part == 0 ? icp_row(ref, cur, l, &T, p, row) : rgb_row(ref, cur, l, &T, TO_R(stddev), p, row);
            if (!ok) continue;
            float *a = t + 29 * part;
            int k = 0;
            for (int i = 0; i < 7; ++i)
                for (int j = i; j < 7; ++j) a[k++] = (float)(row[i] * row[j]);
            a[28] = 1.f;
        }
    }
}

/* FP64 6x6 LDL^T with symmetric diagonal pivoting (documented Eigen::LDLT
 * method, icp_tracker.cpp:92); a zero pivot yields a zero component */
static void ldlt6(double A[6][6], const double b[6], double x[6]) {
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

/* SE(3) exponential, xi = (rho, phi) translation first (Sophus::SE3d::exp) */
static void se3_exp(const double xi[6], double T[12]) {
    const double wx = xi[3], wy = xi[4], wz = xi[5];
    const double th2 = wx * wx + wy * wy + wz * wz, th = sqrt(th2);
    double A, B, C;
    if (th < 1e-5) {
        A = 1.0 - th2 / 6.0; B = 0.5 - th2 / 24.0; C = 1.0 / 6.0 - th2 / 120.0;
    } else {
        const double s = sin(th), c = cos(th);
        A = s / th; B = (1.0 - c) / th2; C = (th - s) / (th2 * th);
    }
    const double W[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    double W2[9], V[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) W2[i * 3 + j] = W[i * 3] * W[j] + W[i * 3 + 1] * W[3 + j] + W[i * 3 + 2] * W[6 + j];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double I = (i == j) ? 1.0 : 0.0;
            T[i * 4 + j] = I + A * W[i * 3 + j] + B * W2[i * 3 + j];
            V[i * 3 + j] = I + B * W[i * 3 + j] + C * W2[i * 3 + j];
        }
    for (int i = 0; i < 3; ++i) T[i * 4 + 3] = V[i * 3] * xi[0] + V[i * 3 + 1] * xi[1] + V[i * 3 + 2] * xi[2];
}

static double se3_log_norm(const double T[12]) {
    const double tr = T[0] + T[5] + T[10];
    double c = (tr - 1.0) * 0.5;
    c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
    const double th = acos(c);
    const double vx = T[9] - T[6], vy = T[2] - T[8], vz = T[4] - T[1];
    double k = 0.5;
    const double s = sin(th);
    if (th > 1e-8 && s > 1e-12) k = th / (2.0 * s);
    const double wx = k * vx, wy = k * vy, wz = k * vz;
    const double th2 = wx * wx + wy * wy + wz * wz;
    double f;
    if (th2 < 1e-10) f = 1.0 / 12.0;
    else {
        const double t = sqrt(th2), A = sin(t) / t, B = (1.0 - cos(t)) / th2;
        f = (1.0 - A / (2.0 * B)) / th2;
    }
    const double W[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    const double t3[3] = {T[3], T[7], T[11]};
    double rho[3];
    for (int i = 0; i < 3; ++i) {
        double r = t3[i];
        for (int j = 0; j < 3; ++j) {
            const double w2 = W[i * 3] * W[j] + W[i * 3 + 1] * W[3 + j] + W[i * 3 + 2] * W[6 + j];
            r += -0.5 * W[i * 3 + j] * t3[j] + f * w2 * t3[j];
        }
        rho[i] = r;
    }
    return sqrt(rho[0] * rho[0] + rho[1] * rho[1] + rho[2] * rho[2] + th2);
}

/* DenseTracking::compute_transform (src/tracking/icp_tracker.cpp:23-156) */
void SFX(or_track)(const FRAME *ref, const FRAME *cur, const double init[16], or_track_result *res) {
    const or_config *c = &ref->cfg;
    double est[12], prev[12], ini[12];
    memcpy(est, init, sizeof(est));
    memcpy(ini, init, sizeof(ini));
    pose_eye(prev);
    int invalid = 0, iterations = 0;
    float icp_e = FLT_MAX, rgb_e = FLT_MAX, n_icp_last = 0, n_rgb_last = 0;
    for (int l = c->num_levels - 1; l >= 0; --l) {
        float icp_error = FLT_MAX, rgb_error = FLT_MAX, stddev = 0;
        int icp_count = 0, rgb_count = 0;
        for (int it = 0; it < c->max_iterations[l]; ++it) {
            double last[12];
            memcpy(last, est, sizeof(last));
            const float last_icp = icp_error, last_rgb = rgb_error;
            float Tf[12];
            for (int i = 0; i < 12; ++i) Tf[i] = (float)last[i];
            double s[58];
            SFX(or_reduce)(ref, cur, l, Tf, stddev, s);
            /* create_jtjjtr (reduce_sum.h:48-61) into float matrices */
            float Hi[6][6], Hr[6][6], bi[6], br[6];
            int k = 0;
            for (int i = 0; i < 6; ++i)
                for (int j = i; j < 7; ++j, ++k) {
                    const float vi = (float)s[k], vr = (float)s[29 + k];
                    if (j == 6) { bi[i] = vi; br[i] = vr; }
                    else { Hi[i][j] = Hi[j][i] = vi; Hr[i][j] = Hr[j][i] = vr; }
                }
            const float r_icp = (float)s[27], n_icp = (float)s[28], r_rgb = (float)s[56], n_rgb = (float)s[57];
            stddev = sqrtf(r_rgb / (n_rgb - 6.0f));
            double A[6][6], b[6], xi[6];
            for (int i = 0; i < 6; ++i) {
                for (int j = 0; j < 6; ++j) A[i][j] = (double)(c->w_icp * Hi[i][j] + c->w_rgb * Hr[i][j]);
                b[i] = (double)(c->w_icp * bi[i] + c->w_rgb * br[i]);
            }
            ldlt6(A, b, xi);
            double E[12], next[12];
            se3_exp(xi, E);
            pose_mul(E, last, next);
            memcpy(prev, est, sizeof(prev));
            memcpy(est, next, sizeof(est));
            iterations++;
            n_icp_last = n_icp;
            n_rgb_last = n_rgb;
            icp_error = sqrtf(r_icp) / n_icp;
            if (isnan(icp_error)) { invalid = 1; break; }
            if (icp_error > last_icp) {
                if (icp_count >= 2) { memcpy(est, prev, sizeof(est)); break; }
                icp_count++;
                icp_error = last_icp;
            } else icp_count = 0;
            rgb_error = sqrtf(r_rgb) / n_rgb;
            if (isnan(rgb_error)) { invalid = 1; break; }
            if (rgb_error > last_rgb) {
                if (rgb_count >= 2) { memcpy(est, prev, sizeof(est)); break; }
                rgb_count++;
                rgb_error = last_rgb;
            } else rgb_count = 0;
        }
        icp_e = icp_error;
        rgb_e = rgb_error;
    }
    double inv[12], rel[12];
    pose_inv(est, inv);
    pose_mul(inv, ini, rel);
    const double n = se3_log_norm(rel);
    int finite = 1;
    for (int i = 0; i < 12; ++i) finite &= isfinite(est[i]) ? 1 : 0;
    const int fail = invalid || !(n <= 0.1) || !finite;
    res->success = !fail;
    res->iterations = iterations;
    res->icp_error = icp_e;
    res->rgb_error = rgb_e;
    res->icp_inliers = n_icp_last;
    res->rgb_inliers = n_rgb_last;
    double up[12];
    if (fail) pose_eye(up);
    else memcpy(up, inv, sizeof(up));
    for (int i = 0; i < 12; ++i) res->update[i] = up[i];
    res->update[12] = res->update[13] = res->update[14] = 0;
    res->update[15] = 1;
}

/* ================================================================== system */

struct SFX(or_system) {
    or_config cfg;
    or_intrinsics K;
    MAP *map;
    FRAME *fr[2];
    int ref, has_ref;
    double pose[12];
    double prior[16];   /* the next frame's initial estimate (gbf_config::motion_prior) */
    or_track_result last;
    float *depth_m, *vmap;
};
typedef struct SFX(or_system) SYS;

SYS *SFX(or_system_create)(const or_config *cfg, const or_intrinsics *K) {
    SYS *s = (SYS *)calloc(1, sizeof(SYS));
    s->cfg = *cfg;
    s->K = *K;
    s->map = SFX(or_map_create)(cfg, K);
    s->fr[0] = SFX(or_frame_create)(cfg, K);
    s->fr[1] = SFX(or_frame_create)(cfg, K);
    pose_eye(s->pose);
    pose_eye(s->prior);
    s->depth_m = (float *)malloc((size_t)K->width * K->height * sizeof(float));
    s->vmap = (float *)malloc((size_t)K->width * K->height * 4 * sizeof(float));
    return s;
}

void SFX(or_system_destroy)(SYS *s) {
    if (!s) return;
    SFX(or_map_destroy)(s->map);
    SFX(or_frame_destroy)(s->fr[0]);
    SFX(or_frame_destroy)(s->fr[1]);
    free(s->depth_m);
    free(s->vmap);
    free(s);
}

void SFX(or_system_set_pose)(SYS *s, const double T[16]) { memcpy(s->pose, T, 12 * sizeof(double)); }

void SFX(or_system_get_pose)(const SYS *s, double T[16]) {
    memcpy(T, s->pose, 12 * sizeof(double));
    T[12] = T[13] = T[14] = 0;
    T[15] = 1;
}

MAP *SFX(or_system_map)(SYS *s) { return s->map; }
FRAME *SFX(or_system_ref)(SYS *s) { return s->fr[s->ref]; }
void SFX(or_system_last_result)(const SYS *s, or_track_result *r) { *r = s->last; }

/* System::process_images (src/system.cpp:40-70) with DenseOdometry::trackFrame
 * (src/tracking/rgbd_odometry.cpp:18-48) */
void SFX(or_process_frame)(SYS *s, const uint16_t *depth_mm, const uint8_t *rgb) {
    const size_t P = (size_t)s->K.width * s->K.height;
    for (size_t i = 0; i < P; ++i) s->depth_m[i] = (float)depth_mm[i] * 0.001f; /* system.cpp:43 */
    const int cur = 1 - s->ref;
    SFX(or_build_pyramid)(s->fr[cur], s->depth_m, rgb);
    if (s->has_ref) {
        SFX(or_track)(s->fr[s->ref], s->fr[cur], s->prior, &s->last);
        double np[12];
        pose_mul(s->pose, s->last.update, np);
        memcpy(s->pose, np, sizeof(np));
    } else {
        memset(&s->last, 0, sizeof(s->last));
        s->last.success = 1;
    }
    /* the next frame starts from no motion (rgbd_odometry.cpp:33-37), or with
     * the constant-velocity prior from the motion this frame tracked */
    if (s->cfg.motion_prior && s->has_ref && s->last.success)
        pose_inv(s->last.update, s->prior);
    else
        pose_eye(s->prior);
    s->ref = cur;
    s->has_ref = 1;
    /* fuse the raw depth with the new frame's level-0 normals (voxel_hashing.cpp:44-65) */
    double T[16];
    SFX(or_system_get_pose)(s, T);
    FRAME *f = s->fr[s->ref];
    float *n0 = (float *)malloc(P * 4 * sizeof(float));
    SFX(or_frame_get)(f, 1, 0, n0);
    SFX(or_fuse)(s->map, s->depth_m, rgb, n0, T);
    free(n0);
    /* raycast into the reference vertex map, then its pyramid (system.cpp:65-66) */
    SFX(or_frame_get)(f, 0, 0, s->vmap);
    SFX(or_raycast)(s->map, T, s->vmap);
    SFX(or_frame_set_vmap)(f, s->vmap);
}
