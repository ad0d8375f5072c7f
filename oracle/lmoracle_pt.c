/*
 * CPU oracle: renderer::pt on diffuse surfaces and area lights.
 *
 * TEST INFRASTRUCTURE ONLY (see lmoracle.h).  Restates, in C:
 *   Renderer_PT sample loop          src/liblightmetrica/renderer/renderer_pt.cpp:68-231
 *   Sensor_Pinhole direction/raster  src/liblightmetrica/asset/sensor/sensor_pinhole.cpp:79-90, 165-185
 *   lookat camera basis              src/liblightmetrica/scene3.cpp:213-221
 *   BSDF_Diffuse sample/evaluate     src/liblightmetrica/asset/bsdf/bsdf_diffuse.cpp:69-104
 *   concentric-disk cosine sampling  include/lightmetrica/sampler.h:44-67
 *   Light_Area emission (front face) src/liblightmetrica/asset/light/light_area.cpp:108-113
 *   hit frame (gn, OrthonormalBasis) include/lightmetrica/intersectionutils.h:78-131, math.h:2355-2359
 *   Film_HDR::Splat pixel index      src/liblightmetrica/asset/film/film_hdr.cpp:218-223
 * Intersections use the oracle's accel::bvh_sahbin (lmoracle_accel.c) with
 * [EpsIsect, Inf] as Scene3::Intersect does (scene3.cpp:458-462).
 *
 * Sampling follows the reference estimator exactly (raster positions uniform
 * over the whole film, Russian roulette 0.5 at every bounce), with its own
 * random number generator (splitmix64 per thread): results agree with the
 * reference statistically, not sample by sample.  Films are accumulated in
 * double together with per-pixel sums of squares.
 */
#include "lmoracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.14159265358979323846f

static inline uint64_t splitmix64(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline float rnd(uint64_t* s) { return (float)(splitmix64(s) >> 40) * (1.0f / 16777216.0f); }

typedef struct { float x, y, z; } v3;
static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) { return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
static inline v3 normalize(v3 a) { return mul(a, 1.0f / sqrtf(dot(a, a))); }

typedef struct {
    const lmo_accel* accel;
    const float* tris;
    const int32_t* tri_prim;
    const lmo_pt_prim* prims;
    lmo_pt_camera cam;
    v3 vx, vy, vz, eye;
    float tan_fov, aspect;
    uint64_t num_samples;
    int max_num_vertices;
    uint64_t seed;
    int threads;
    double* sum;   /* shared output, merged under the lock */
    double* sumsq;
    pthread_mutex_t lock;
} pt_job;

typedef struct {
    pt_job* job;
    int index;
} pt_worker;

/* Sampler::UniformConcentricDiskSample + CosineSampleHemisphere (sampler.h:44-67) */
static v3 cosine_hemisphere(float u0, float u1)
{
    float vx = 2.0f * u0 - 1.0f, vy = 2.0f * u1 - 1.0f;
    float sx = 0.0f, sy = 0.0f;
    if (!(vx == 0.0f && vy == 0.0f)) {
        float r, theta;
        if (vx > -vy) {
            if (vx > vy) { r = vx; theta = (PI_F * 0.25f) * vy / vx; }
            else { r = vy; theta = (PI_F * 0.25f) * (2.0f - vx / vy); }
        } else {
            if (vx < vy) { r = -vx; theta = (PI_F * 0.25f) * (4.0f + vy / vx); }
            else { r = -vy; theta = (PI_F * 0.25f) * (6.0f - vx / vy); }
        }
        sx = r * cosf(theta);
        sy = r * sinf(theta);
    }
    float z2 = 1.0f - sx * sx - sy * sy;
    return V(sx, sy, sqrtf(z2 > 0.0f ? z2 : 0.0f));
}

/* Math::OrthonormalBasis (math.h:2355-2359): ToWorld = (b, c, a) columns. */
static void basis(v3 a, v3* b, v3* c)
{
    *c = fabsf(a.x) > fabsf(a.y) ? normalize(V(a.z, 0.0f, -a.x)) : normalize(V(0.0f, a.z, -a.y));
    *b = cross(*c, a);
}

static void* pt_worker_fn(void* arg)
{
    pt_worker* w = (pt_worker*)arg;
    pt_job* J = w->job;
    const int W = J->cam.width, H = J->cam.height;
    double* sum = (double*)calloc((size_t)W * H * 3, sizeof(double));
    double* sumsq = (double*)calloc((size_t)W * H * 3, sizeof(double));
    /* independent stream per worker: hash (seed, worker) into the state */
    uint64_t rng = J->seed ^ 0xD1B54A32D192ED03ull;
    rng = splitmix64(&rng) ^ ((uint64_t)w->index * 0xA0761D6478BD642Full);
    rng = splitmix64(&rng);
    const uint64_t b = J->num_samples * (uint64_t)w->index / (uint64_t)J->threads;
    const uint64_t e = J->num_samples * (uint64_t)(w->index + 1) / (uint64_t)J->threads;
    for (uint64_t s = b; s < e; s++) {
        /* sensor: raster position uniform over the film (sensor_pinhole.cpp:79-90) */
        const float u0 = rnd(&rng), u1 = rnd(&rng);
        const float rx = 2.0f * u0 - 1.0f, ry = 2.0f * u1 - 1.0f;
        const v3 we = normalize(V(J->aspect * J->tan_fov * rx, J->tan_fov * ry, -1.0f));
        v3 d = add(add(mul(J->vx, we.x), mul(J->vy, we.y)), mul(J->vz, we.z));
        /* raster position from the direction (sensor_pinhole.cpp:165-185) */
        const float ex = dot(J->vx, d), ey = dot(J->vy, d), ez = dot(J->vz, d);
        if (ez >= 0.0f) continue;
        const float px = (-ex / ez / J->tan_fov / J->aspect + 1.0f) * 0.5f;
        const float py = (-ey / ez / J->tan_fov + 1.0f) * 0.5f;
        if (px < 0.0f || px > 1.0f || py < 0.0f || py > 1.0f) continue;
        int ix = (int)(px * (float)W), iy = (int)(py * (float)H);
        ix = ix < 0 ? 0 : (ix > W - 1 ? W - 1 : ix);
        iy = iy < 0 ? 0 : (iy > H - 1 ? H - 1 : iy);
        const size_t pix = (size_t)iy * W + ix;

        v3 thr = V(1.0f, 1.0f, 1.0f);
        v3 o = J->eye;
        int nv = 1;
        for (;;) {
            if (J->max_num_vertices != -1 && nv >= J->max_num_vertices) break;
            float ray[8] = {o.x, o.y, o.z, 1e-4f, d.x, d.y, d.z, FLT_MAX};
            lmo_hit h;
            lmo_accel_trace(J->accel, ray, 1, &h, 1);
            if (h.id < 0) break;
            const float* T = J->tris + 9 * (size_t)h.id;
            const v3 p1 = V(T[0], T[1], T[2]), p2 = V(T[3], T[4], T[5]), p3 = V(T[6], T[7], T[8]);
            const v3 gn = normalize(cross(sub(p2, p1), sub(p3, p1)));
            const lmo_pt_prim* P = &J->prims[J->tri_prim[h.id]];
            const v3 p = V(h.p[0], h.p[1], h.p[2]);
            if (P->is_light) {
                /* Le only on the front side (light_area.cpp:108-113) */
                if (dot(mul(d, -1.0f), gn) > 0.0f) {
                    const float c[3] = {thr.x * P->Le[0], thr.y * P->Le[1], thr.z * P->Le[2]};
                    for (int k = 0; k < 3; k++) {
                        sum[3 * pix + k] += c[k];
                        sumsq[3 * pix + k] += (double)c[k] * (double)c[k];
                    }
                }
            }
            /* Russian roulette (renderer_pt.cpp:207-216) */
            if (rnd(&rng) > 0.5f) break;
            thr = mul(thr, 2.0f);
            nv++;
            if (J->max_num_vertices != -1 && nv >= J->max_num_vertices) break;
            if (P->bsdf != LMO_BSDF_DIFFUSE) break; /* bsdf::null: black, path ends */
            /* bsdf::diffuse (bsdf_diffuse.cpp:69-104), sn = gn (no vertex normals) */
            const v3 wi = mul(d, -1.0f);
            if (dot(wi, gn) <= 0.0f) break;
            v3 bx, by;
            basis(gn, &bx, &by);
            const float a0 = rnd(&rng), a1 = rnd(&rng);
            const v3 lw = cosine_hemisphere(a0, a1);
            if (lw.z <= 0.0f) break;
            const v3 wo = add(add(mul(bx, lw.x), mul(by, lw.y)), mul(gn, lw.z));
            if (dot(wo, gn) <= 0.0f) break;
            thr = V(thr.x * P->R[0], thr.y * P->R[1], thr.z * P->R[2]);
            o = p;
            d = wo;
        }
    }
    pthread_mutex_lock(&J->lock);
    for (size_t i = 0; i < (size_t)W * H * 3; i++) { J->sum[i] += sum[i]; J->sumsq[i] += sumsq[i]; }
    pthread_mutex_unlock(&J->lock);
    free(sum);
    free(sumsq);
    return NULL;
}

uint64_t lmo_render_pt(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                       const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices, uint64_t seed,
                       int threads, double* sum, double* sumsq)
{
    pt_job J;
    memset(&J, 0, sizeof(J));
    J.accel = lmo_accel_build(1, tris, ntri);
    J.tris = tris;
    J.tri_prim = tri_prim;
    J.prims = prims;
    J.cam = *cam;
    J.eye = V(cam->eye[0], cam->eye[1], cam->eye[2]);
    const v3 c = V(cam->center[0], cam->center[1], cam->center[2]);
    const v3 up = V(cam->up[0], cam->up[1], cam->up[2]);
    J.vz = normalize(sub(J.eye, c));
    J.vx = normalize(cross(up, J.vz));
    J.vy = cross(J.vz, J.vx);
    J.tan_fov = tanf(cam->fov_deg * PI_F / 180.0f * 0.5f);
    J.aspect = (float)cam->width / (float)cam->height;
    J.num_samples = num_samples;
    J.max_num_vertices = max_num_vertices;
    J.seed = seed;
    J.threads = threads < 1 ? 1 : threads;
    J.sum = sum;
    J.sumsq = sumsq;
    memset(sum, 0, sizeof(double) * (size_t)cam->width * cam->height * 3);
    memset(sumsq, 0, sizeof(double) * (size_t)cam->width * cam->height * 3);
    pthread_mutex_init(&J.lock, NULL);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)J.threads);
    pt_worker* ws = (pt_worker*)malloc(sizeof(pt_worker) * (size_t)J.threads);
    for (int i = 0; i < J.threads; i++) {
        ws[i].job = &J;
        ws[i].index = i;
        pthread_create(&th[i], NULL, pt_worker_fn, &ws[i]);
    }
    for (int i = 0; i < J.threads; i++) pthread_join(th[i], NULL);
    pthread_mutex_destroy(&J.lock);
    free(th);
    free(ws);
    lmo_accel_free((lmo_accel*)J.accel);
    return num_samples;
}
