/*
 * CPU oracle: renderer::pt on diffuse surfaces and area lights.
 *
 * TEST INFRASTRUCTURE ONLY (see lmoracle.h).  Restates, in C:
 *   Renderer_PT sample loop          src/liblightmetrica/renderer/renderer_pt.cpp:68-231
 *   Sensor_Pinhole direction/raster  src/liblightmetrica/asset/sensor/sensor_pinhole.cpp:79-90, 165-185
 *   lookat camera basis              src/liblightmetrica/scene3.cpp:213-221
 *   BSDF_Diffuse sample/evaluate     src/liblightmetrica/asset/bsdf/bsdf_diffuse.cpp:69-104
 *   concentric-disk cosine sampling  include/lightmetrica/sampler.h:44-67
 *   BSDF_Flesnel sample/evaluate     src/liblightmetrica/asset/bsdf/bsdf_flesnel.cpp:59-164, 225-241
 *   BSDF_CookTorrance (GGX)          src/liblightmetrica/asset/bsdf/bsdf_cooktorrance.cpp:73-292
 *   Light_Area emission (front face) src/liblightmetrica/asset/light/light_area.cpp:108-113
 *   Light_EnvLight (constant Le) on the scene's bounding sphere, hit when
 *   the accel misses            light_env.cpp:42-230, scene3.cpp:52-78, 464-475
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
    lmo_pt_env env;
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

/* BSDF_Flesnel::EvaluateFresnelTerm (bsdf_flesnel.cpp:243-257) */
static float fresnel_dielectric(float wiDotN, float etaI, float etaT)
{
    const float eta = etaI / etaT;
    const float cosThetaTSq = 1.0f - eta * eta * (1.0f - wiDotN * wiDotN);
    if (cosThetaTSq <= 0.0f) return 1.0f;
    const float ci = fabsf(wiDotN), ct = sqrtf(cosThetaTSq);
    const float rs = (etaI * ci - etaT * ct) / (etaI * ci + etaT * ct);
    const float rt = (etaI * ct - etaT * ci) / (etaI * ct + etaT * ci);
    return (rs * rs + rt * rt) * 0.5f;
}

/* BSDF_CookTorrance::EvaluateGGX (bsdf_cooktorrance.cpp:187-198) */
static float ggx_d(v3 H, float a)
{
    const float c = H.z;
    if (c <= 0.0f) return 0.0f;
    const float t = 1.0f - c * c;
    const float tanH = t <= 0.0f ? 0.0f : sqrtf(t) / c;
    const float q = a * a + tanH * tanH;
    return (a * a) / (PI_F * c * c * c * c * q * q);
}

/* BSDF_CookTorrance::SampleGGX (bsdf_cooktorrance.cpp:200-225), Eps = 1e-4 */
static v3 ggx_sample(float ua, float ub, float a)
{
    const float eps = 1e-4f;
    const float u0 = (1.0f - eps) * ua + eps;
    const float u1 = (1.0f - 2.0f * eps) * ub + eps;
    const float den = sqrtf(1.0f - (1.0f - a * a) * u0);
    const float cosT = sqrtf(1.0f - u0) / den;
    const float sinT = a * (sqrtf(u0) / den);
    const float phi = PI_F * (2.0f * u1 - 1.0f);
    return V(sinT * cosf(phi), sinT * sinf(phi), cosT);
}

/* BSDF_CookTorrance::EvaluateFrConductor (bsdf_cooktorrance.cpp:283-291), one channel */
static float fresnel_conductor(float c, float eta, float k)
{
    const float tmp = (eta * eta + k * k) * (c * c);
    const float rParl2 = (tmp - (eta * (2.0f * c)) + 1.0f) / (tmp + (eta * (2.0f * c)) + 1.0f);
    const float tmpF = eta * eta + k * k;
    const float rPerp2 = (tmpF - (eta * (2.0f * c)) + c * c) / (tmpF + (eta * (2.0f * c)) + c * c);
    return (rParl2 + rPerp2) * 0.5f;
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
            if (h.id < 0) {
                /* the environment's bounding sphere contains every vertex and
                 * the sensor, so a ray leaving the geometry always meets it */
                if (J->env.enabled) {
                    const float c[3] = {thr.x * J->env.Le[0], thr.y * J->env.Le[1], thr.z * J->env.Le[2]};
                    for (int k = 0; k < 3; k++) {
                        sum[3 * pix + k] += c[k];
                        sumsq[3 * pix + k] += (double)c[k] * (double)c[k];
                    }
                }
                break;
            }
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
            if (P->bsdf == LMO_BSDF_NULL) break; /* bsdf::null: black, path ends */
            /* shading frame: sn = gn (no vertex normals), OrthonormalBasis */
            const v3 wi = mul(d, -1.0f);
            v3 bx, by;
            basis(gn, &bx, &by);
            const v3 lwi = V(dot(wi, bx), dot(wi, by), dot(wi, gn));
            const float a0 = rnd(&rng), a1 = rnd(&rng), a2 = rnd(&rng);
            v3 lwo;
            float f[3];
            if (P->bsdf == LMO_BSDF_DIFFUSE) {
                /* bsdf_diffuse.cpp:69-104: fs / pdf = R */
                if (lwi.z <= 0.0f) break;
                lwo = cosine_hemisphere(a0, a1);
                if (lwo.z <= 0.0f) break;
                for (int k = 0; k < 3; k++) f[k] = P->R[k];
            } else if (P->bsdf == LMO_BSDF_DIELECTRIC) {
                /* bsdf_flesnel.cpp:59-164: reflect w.p. Fr, else refract;
                 * fs / pdf = R, or R * (etaI / etaT)^2 for refraction (EL) */
                float etaI = P->eta1, etaT = P->eta2;
                if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
                const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
                float scale = 1.0f;
                if (a2 <= Fr) {
                    lwo = V(-lwi.x, -lwi.y, lwi.z);
                } else {
                    const float eta = etaI / etaT;
                    const float cosTSq = 1.0f - eta * eta * (1.0f - lwi.z * lwi.z);
                    const float cosT = sqrtf(cosTSq > 0.0f ? cosTSq : 0.0f) * (lwi.z > 0.0f ? -1.0f : 1.0f);
                    lwo = V(-eta * lwi.x, -eta * lwi.y, cosT);
                    scale = eta * eta;
                }
                for (int k = 0; k < 3; k++) f[k] = P->R[k] * scale;
            } else {
                /* bsdf_cooktorrance.cpp:73-120 (GGX):
                 * fs / pdf = R D G F / (4 cos_i cos_o) / (D cos_H / (4 (wo.H)) / cos_o) */
                if (lwi.z <= 0.0f) break;
                const v3 H = ggx_sample(a0, a1, P->roughness);
                const float dih = dot(mul(lwi, -1.0f), H);
                lwo = sub(mul(lwi, -1.0f), mul(H, 2.0f * dih));
                if (lwo.z <= 0.0f) break;
                const v3 Hn = normalize(add(lwi, lwo));
                const float D = ggx_d(Hn, P->roughness);
                const float woH = fabsf(dot(lwo, Hn));
                const float G1 = 2.0f * Hn.z * lwo.z / woH, G2 = 2.0f * Hn.z * lwi.z / woH;
                const float G = fminf(1.0f, fminf(G1, G2));
                const float pdf = D * Hn.z / (4.0f * dot(lwo, Hn)) / lwo.z;
                if (!(pdf > 0.0f)) break;
                for (int k = 0; k < 3; k++) {
                    const float F = fresnel_conductor(dot(lwi, Hn), P->ct_eta[k], P->ct_k[k]);
                    const float fs = P->R[k] * D * G * F / (4.0f * lwi.z) / lwo.z;
                    f[k] = fs / pdf;
                }
            }
            if (f[0] == 0.0f && f[1] == 0.0f && f[2] == 0.0f) break;
            const v3 wo = add(add(mul(bx, lwo.x), mul(by, lwo.y)), mul(gn, lwo.z));
            thr = V(thr.x * f[0], thr.y * f[1], thr.z * f[2]);
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
                       const lmo_pt_env* env, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                       uint64_t seed, int threads, double* sum, double* sumsq)
{
    pt_job J;
    memset(&J, 0, sizeof(J));
    if (env) J.env = *env;
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
