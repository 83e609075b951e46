// synth.cu -- seeded synthetic RGB-D scenes: a box room with spheres and
// axis-aligned boxes, sphere-traced into u16 depth (mm) + rgb8 with a
// procedural texture and the depth noise model sigma(z) = 0.0012 + 0.0019 (z - 0.4)^2.
// These stand in for the reference's camera input (OpenNI DEPTH_1_MM + RGB888,
// src/input/oni_camera.cpp:44-48); no dataset is available on either machine.
#include <math.h>
#include <stdlib.h>

#include <new>
#include <vector>

#include "gbf_internal.h"

namespace gbf {

namespace {

constexpr int kMaxPrims = 48;

struct SceneDev {
    float room[3];
    int ns, nb;
    float4 sph[kMaxPrims];   // centre, radius
    float4 boxc[kMaxPrims];  // centre
    float4 boxh[kMaxPrims];  // half extent
    float4 tint[2 * kMaxPrims + 1];
    unsigned long long seed;
    float noise, zmin, zmax;
};

__host__ __device__ inline unsigned long long splitmix(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ inline float box_sdf(float3 p, float4 c, float4 h) {
    const float qx = fabsf(p.x - c.x) - h.x, qy = fabsf(p.y - c.y) - h.y, qz = fabsf(p.z - c.z) - h.z;
    const float ox = fmaxf(qx, 0.f), oy = fmaxf(qy, 0.f), oz = fmaxf(qz, 0.f);
    return sqrtf(ox * ox + oy * oy + oz * oz) + fminf(fmaxf(qx, fmaxf(qy, qz)), 0.f);
}

// scene distance; id 0 = room, 1..ns spheres, ns+1.. boxes
__device__ inline float scene_sdf(const SceneDev &s, float3 p, int &id) {
    float d = fminf(fminf(fminf(p.x, s.room[0] - p.x), fminf(p.y, s.room[1] - p.y)), fminf(p.z, s.room[2] - p.z));
    id = 0;
    for (int i = 0; i < s.ns; ++i) {
        const float4 c = s.sph[i];
        const float dx = p.x - c.x, dy = p.y - c.y, dz = p.z - c.z;
        const float e = sqrtf(dx * dx + dy * dy + dz * dz) - c.w;
        if (e < d) { d = e; id = 1 + i; }
    }
    for (int i = 0; i < s.nb; ++i) {
        const float e = box_sdf(p, s.boxc[i], s.boxh[i]);
        if (e < d) { d = e; id = 1 + s.ns + i; }
    }
    return d;
}

__global__ void render_kernel(SceneDev s, gbf_intrinsics K, M34Host T, int frame, uint16_t *depth, uint8_t *rgb) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= K.width || y >= K.height) return;
    const float dcx = ((float)x - K.cx) / K.fx, dcy = ((float)y - K.cy) / K.fy;
    const float dl = sqrtf(dcx * dcx + dcy * dcy + 1.f);
    const float3 dir = make_float3((T.m[0] * dcx + T.m[1] * dcy + T.m[2]) / dl, (T.m[4] * dcx + T.m[5] * dcy + T.m[6]) / dl,
                                   (T.m[8] * dcx + T.m[9] * dcy + T.m[10]) / dl);
    const float3 o = make_float3(T.m[3], T.m[7], T.m[11]);
    float t = 0.05f;
    int id = 0;
    bool hit = false;
    for (int i = 0; i < 256 && t < 20.f; ++i) {
        const float3 p = make_float3(o.x + dir.x * t, o.y + dir.y * t, o.z + dir.z * t);
        const float d = scene_sdf(s, p, id);
        if (d < 1e-4f * t + 2e-5f) { hit = true; break; }
        t += d;
    }
    const size_t pix = (size_t)y * K.width + x;
    float z = hit ? t / dl : 0.f;
    unsigned char cr = 0, cg = 0, cb = 0;
    if (hit) {
        const float3 p = make_float3(o.x + dir.x * t, o.y + dir.y * t, o.z + dir.z * t);
        const float e = 1e-3f;
        int dummy;
        float3 n = make_float3(scene_sdf(s, make_float3(p.x + e, p.y, p.z), dummy) - scene_sdf(s, make_float3(p.x - e, p.y, p.z), dummy),
                               scene_sdf(s, make_float3(p.x, p.y + e, p.z), dummy) - scene_sdf(s, make_float3(p.x, p.y - e, p.z), dummy),
                               scene_sdf(s, make_float3(p.x, p.y, p.z + e), dummy) - scene_sdf(s, make_float3(p.x, p.y, p.z - e), dummy));
        const float nl = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z) + 1e-12f;
        n = make_float3(n.x / nl, n.y / nl, n.z / nl);
        const float3 L = make_float3(0.32f, 0.48f, 0.82f);
        const float lam = 0.35f + 0.65f * fmaxf(0.f, n.x * L.x + n.y * L.y + n.z * L.z);
        // view-independent texture: smooth stripes of several frequencies
        const float pat = 0.5f + 0.22f * sinf(23.1f * p.x + 5.f * sinf(7.3f * p.y)) +
                          0.18f * sinf(19.7f * p.y + 17.3f * p.z + 3.f * cosf(5.1f * p.x)) +
                          0.10f * sinf(41.0f * p.z - 29.0f * p.x);
        const float4 tint = s.tint[id];
        const float a = fminf(fmaxf(lam * (0.35f + 0.65f * pat), 0.f), 1.f) * 255.f;
        cr = (unsigned char)fminf(a * tint.x, 255.f);
        cg = (unsigned char)fminf(a * tint.y, 255.f);
        cb = (unsigned char)fminf(a * tint.z, 255.f);
        if (s.noise > 0.f) {
            const unsigned long long h = splitmix(s.seed ^ splitmix(((unsigned long long)frame << 32) ^ (unsigned long long)pix));
            const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.f);
            const float u2 = ((float)((h >> 16) & 0xFFFFFF) + 0.5f) * (1.0f / 16777216.f);
            const float g = sqrtf(-2.f * logf(u1)) * cosf(6.2831853f * u2);
            const float sg = 0.0012f + 0.0019f * (z - 0.4f) * (z - 0.4f);
            z += s.noise * sg * g;
        }
        if (z < s.zmin || z > s.zmax) z = 0.f;
    }
    depth[pix] = (uint16_t)(z > 0.f ? fminf(rintf(z * 1000.f), 65535.f) : 0.f);
    rgb[pix * 3 + 0] = cr;
    rgb[pix * 3 + 1] = cg;
    rgb[pix * 3 + 2] = cb;
}

double urand(unsigned long long &st) {
    st = splitmix(st);
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

struct SynthScene {
    gbf_synth_params p;
    SceneDev dev;
    std::vector<double> path_s;  // figure-eight arc-length table
};

// camera position + forward direction at frame k
static void path_at(const SynthScene &sc, int k, double pos[3], double fwd[3]) {
    const gbf_synth_params &p = sc.p;
    const double cx = p.room[0] * 0.5, cy = p.room[1] * 0.5;
    const double jitter = p.yaw_jitter_deg * M_PI / 180.0 * sin(2.0 * M_PI * k / 150.0 + 0.7);  // smooth, 5 s period
    double yaw;
    if (p.trajectory == 0) {
        const double th = 2.0 * M_PI * k / (p.frames_per_loop > 0 ? p.frames_per_loop : 200);
        pos[0] = cx + p.radius * cos(th);
        pos[1] = cy + p.radius * sin(th);
        pos[2] = p.height;
        yaw = atan2(cy - pos[1], cx - pos[0]) + jitter;  // look at the room centre
    } else {
        // lemniscate of Gerono, constant speed via the arc-length table
        const double s_target = p.speed * k / p.fps;
        const std::vector<double> &tab = sc.path_s;
        const int n = (int)tab.size() - 1;
        const double total = tab[n];
        const double s = fmod(s_target, total);
        int lo = 0, hi = n;
        while (hi - lo > 1) {
            const int mid = (lo + hi) / 2;
            if (tab[mid] <= s) lo = mid; else hi = mid;
        }
        const double f = (tab[hi] > tab[lo]) ? (s - tab[lo]) / (tab[hi] - tab[lo]) : 0.0;
        const double t = 2.0 * M_PI * (lo + f) / n;
        const double a = p.radius;
        pos[0] = cx + a * sin(t);
        pos[1] = cy + a * sin(t) * cos(t);
        pos[2] = p.height;
        const double dx = a * cos(t), dy = a * cos(2.0 * t);
        yaw = atan2(dy, dx) + jitter;
    }
    const double pitch = -10.0 * M_PI / 180.0;
    fwd[0] = cos(pitch) * cos(yaw);
    fwd[1] = cos(pitch) * sin(yaw);
    fwd[2] = sin(pitch);
}

static double dist_to_path(const SynthScene &sc, double x, double y, double z) {
    double best = 1e30;
    for (int k = 0; k < 512; ++k) {
        double pos[3], f[3];
        const int frame = (sc.p.trajectory == 0) ? k * (sc.p.frames_per_loop > 0 ? sc.p.frames_per_loop : 200) / 512
                                                 : (int)(k * (sc.path_s.back() / sc.p.speed * sc.p.fps) / 512);
        path_at(sc, frame, pos, f);
        const double d = sqrt((pos[0] - x) * (pos[0] - x) + (pos[1] - y) * (pos[1] - y) + (pos[2] - z) * (pos[2] - z));
        if (d < best) best = d;
    }
    return best;
}

}  // namespace gbf

using namespace gbf;

struct gbf_synth_scene : public SynthScene {};

extern "C" {

GBF_API gbf_status gbf_synth_default(gbf_synth_params *p) {
    if (!p) return set_error(GBF_ERR_INVALID_ARG, "gbf_synth_default: null");
    gbf_synth_params d{};
    d.room[0] = 4.f; d.room[1] = 4.f; d.room[2] = 3.f;
    d.n_spheres = 6; d.n_boxes = 4;
    d.sphere_rmin = 0.2f; d.sphere_rmax = 0.5f;
    d.seed = 0;
    d.trajectory = 0;
    d.radius = 1.5f; d.height = 1.4f; d.yaw_jitter_deg = 10.f; d.speed = 0.5f; d.fps = 30.f;
    d.frames_per_loop = 600;  // 0.47 m/s at 30 fps on the 1.5 m circle
    d.noise = 1.f;
    d.zclip_min = 0.3f; d.zclip_max = 4.0f;
    *p = d;
    return GBF_OK;
}

GBF_API gbf_status gbf_synth_create(const gbf_synth_params *p, gbf_synth_scene **out) {
    if (!p || !out) return set_error(GBF_ERR_INVALID_ARG, "gbf_synth_create: null");
    if (p->n_spheres < 0 || p->n_spheres > kMaxPrims || p->n_boxes < 0 || p->n_boxes > kMaxPrims)
        return set_error(GBF_ERR_INVALID_ARG, "gbf_synth_create: at most 48 spheres and 48 boxes");
    gbf_synth_scene *sc = new (std::nothrow) gbf_synth_scene();
    if (!sc) return set_error(GBF_ERR_OUT_OF_MEMORY, "gbf_synth_create: host allocation");
    sc->p = *p;
    if (p->trajectory == 1) {
        const int n = 4096;
        sc->path_s.assign(n + 1, 0.0);
        for (int i = 1; i <= n; ++i) {
            const double t0 = 2.0 * M_PI * (i - 1) / n, t1 = 2.0 * M_PI * i / n, a = p->radius;
            const double dx = a * sin(t1) - a * sin(t0), dy = a * sin(t1) * cos(t1) - a * sin(t0) * cos(t0);
            sc->path_s[i] = sc->path_s[i - 1] + sqrt(dx * dx + dy * dy);
        }
    }
    SceneDev &s = sc->dev;
    memset(&s, 0, sizeof(s));
    for (int i = 0; i < 3; ++i) s.room[i] = p->room[i];
    unsigned long long st = splitmix(p->seed * 0x9E37ull + 12345ull);
    const double margin = 0.55;  // keep every object this far from the camera path
    int ns = 0;
    for (int tries = 0; ns < p->n_spheres && tries < 4000; ++tries) {
        const double r = p->sphere_rmin + (p->sphere_rmax - p->sphere_rmin) * urand(st);
        const double x = r + 0.05 + (p->room[0] - 2 * r - 0.1) * urand(st);
        const double y = r + 0.05 + (p->room[1] - 2 * r - 0.1) * urand(st);
        const double z = r + (1.9 - r) * urand(st);
        if (dist_to_path(*sc, x, y, z) < r + margin) continue;
        s.sph[ns++] = make_float4((float)x, (float)y, (float)z, (float)r);
    }
    s.ns = ns;
    int nb = 0;
    for (int tries = 0; nb < p->n_boxes && tries < 4000; ++tries) {
        const double hx = 0.12 + 0.28 * urand(st), hy = 0.12 + 0.28 * urand(st), hz = 0.15 + 0.45 * urand(st);
        const double x = hx + 0.05 + (p->room[0] - 2 * hx - 0.1) * urand(st);
        const double y = hy + 0.05 + (p->room[1] - 2 * hy - 0.1) * urand(st);
        const double z = hz;  // resting on the floor
        const double rr = sqrt(hx * hx + hy * hy + hz * hz);
        if (dist_to_path(*sc, x, y, z) < rr + margin) continue;
        s.boxc[nb] = make_float4((float)x, (float)y, (float)z, 0.f);
        s.boxh[nb] = make_float4((float)hx, (float)hy, (float)hz, 0.f);
        ++nb;
    }
    s.nb = nb;
    for (int i = 0; i < 2 * kMaxPrims + 1; ++i) {
        const float a = 0.55f + 0.45f * (float)urand(st), b = 0.55f + 0.45f * (float)urand(st),
                    c = 0.55f + 0.45f * (float)urand(st);
        s.tint[i] = make_float4(a, b, c, 0.f);
    }
    s.seed = splitmix(p->seed + 777ull);
    s.noise = p->noise;
    s.zmin = p->zclip_min;
    s.zmax = p->zclip_max;
    *out = sc;
    return GBF_OK;
}

GBF_API gbf_status gbf_synth_destroy(gbf_synth_scene *sc) {
    delete sc;
    return GBF_OK;
}

GBF_API gbf_status gbf_synth_pose(const gbf_synth_scene *sc, int32_t frame, double T[16]) {
    if (!sc || !T) return set_error(GBF_ERR_INVALID_ARG, "gbf_synth_pose: null");
    double pos[3], f[3];
    path_at(*sc, frame, pos, f);
    // camera axes in the world: x right = f x up, y down = f x right, z forward = f
    const double up[3] = {0, 0, 1};
    double r[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    const double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int i = 0; i < 3; ++i) r[i] /= rl;
    const double d[3] = {f[1] * r[2] - f[2] * r[1], f[2] * r[0] - f[0] * r[2], f[0] * r[1] - f[1] * r[0]};
    for (int i = 0; i < 3; ++i) {
        T[i * 4 + 0] = r[i];
        T[i * 4 + 1] = d[i];
        T[i * 4 + 2] = f[i];
        T[i * 4 + 3] = pos[i];
    }
    T[12] = T[13] = T[14] = 0.0;
    T[15] = 1.0;
    return GBF_OK;
}

GBF_API gbf_status gbf_synth_render(const gbf_synth_scene *sc, const gbf_intrinsics *K, const double T[16],
                                    int32_t frame, uint16_t *depth, uint8_t *rgb, void *stream) {
    if (!sc || !K || !T || !depth || !rgb) return set_error(GBF_ERR_INVALID_ARG, "gbf_synth_render: null");
    if (K->width <= 0 || K->height <= 0) return set_error(GBF_ERR_INVALID_ARG, "gbf_synth_render: bad size");
    M34Host m;
    for (int i = 0; i < 12; ++i) m.m[i] = (float)T[i];
    dim3 blk(16, 16), grd((K->width + 15) / 16, (K->height + 15) / 16);
    render_kernel<<<grd, blk, 0, (cudaStream_t)stream>>>(sc->dev, *K, m, frame, depth, rgb);
    return check_cuda("gbf_synth_render");
}

}  // extern "C"
