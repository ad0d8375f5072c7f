/*
 * CPU oracle: renderer::bdpt (bidirectional path tracing, power heuristic)
 * and renderer::ptmis (path tracing with next-event estimation and the
 * balance heuristic), which share the surface interactions below.
 *
 * TEST INFRASTRUCTURE ONLY (see lmoracle.h).  Restates, in C, the estimator
 * of src/liblightmetrica/renderer/renderer_bdpt.cpp:
 *   Subpath::Sample                 :80-220  light / eye subpaths; every step
 *                                   after the first stores a BSDF-sampled
 *                                   vertex and a "direct" vertex (the other
 *                                   end's emitter sampled from the previous
 *                                   vertex, kept only if visible); roulette
 *                                   0.5 after each step
 *   Path::Connect                   :233-333
 *   EvaluateUnweightContribution    :489-591  alphaL * Cst * alphaE
 *   EvaluateCst                     :375-406
 *   Samplable / EvaluatePDF         :593-703
 *   MISWeight_PowerHeuristics       :747-784
 *   SelectionPDF                    :348-368  0.5^(max(0,s-2) + max(0,t-2))
 *   Render (strategy loop)          :867-971
 * with the surface interactions it calls:
 *   Light_Area          light_area.cpp:47-127 (SamplePositionAndDirection
 *                       draws the direction from the same 2D sample as the
 *                       position -- replicated), TriangleUtils::SampleTriangleMesh
 *                       triangleutils.h:79-120, Distribution1D::SampleReuse dist.h:71-77
 *   Sensor_Pinhole      sensor_pinhole.cpp:79-202 (delta position; importance
 *                       1 / (4 tan^2 aspect cos^3))
 *   BSDF_Diffuse, BSDF_Flesnel (delta direction), BSDF_CookTorrance, BSDF_Null
 *   GeometryTerm        renderutils.h:46-56; PDFVal conversions probability.h:55-110
 * renderer::ptmis (src/liblightmetrica/renderer/renderer_ptmis.cpp:68-305):
 *   at every vertex before the BSDF sample (the sensor included), one light
 *   sample (primitive uniform, area-CDF triangle, uniform point), weighted
 *   pdf_light / (pdf_light + pdf_bsdf) in projected solid angle (:133-190);
 *   BSDF-sampled light hits weighted pdf_bsdf / (pdf_bsdf + pdf_light), with
 *   pdf_light = 0 after a specular vertex (:246-270); roulette 0.5 (:285-293).
 * renderer::ptdirect (renderer_ptdirect.cpp:72-291): the same light samples
 *   with weight 1, and no emission counted on BSDF-sampled hits.
 * renderer::ltdirect (renderer_ltdirect.cpp:72-279): light paths connected to
 *   the sensor at every vertex with weight 1, roulette 0.5 after each hit.
 * Scene3::Intersect / Visible through the oracle's accel::bvh_sahbin.
 * Environment lights are not part of this restatement.
 */
#include "lmoracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.14159265358979323846f
#define EPS_ISECT 1e-4f

/* SurfaceInteractionType (surfaceinteraction.h:39-52) */
enum { T_D = 1, T_G = 2, T_S = 4, T_L = 8, T_E = 16 };
enum { DIR_LE = 0, DIR_EL = 1 };

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
static inline v3 zero3(void) { return V(0.0f, 0.0f, 0.0f); }

typedef struct { float c[3]; } spd;
static inline spd S1(float v) { spd r = {{v, v, v}}; return r; }
static inline spd S3(const float* v) { spd r = {{v[0], v[1], v[2]}}; return r; }
static inline spd smul(spd a, spd b) { spd r = {{a.c[0] * b.c[0], a.c[1] * b.c[1], a.c[2] * b.c[2]}}; return r; }
static inline spd sscale(spd a, float s) { spd r = {{a.c[0] * s, a.c[1] * s, a.c[2] * s}}; return r; }
static inline int sblack(spd a) { return a.c[0] == 0.0f && a.c[1] == 0.0f && a.c[2] == 0.0f; }

/* A path vertex (PathVertex, renderer_bdpt.cpp:57-62): geometry (sn = gn), the
 * primitive (-1 = the sensor) and the interaction type it plays. */
typedef struct {
    v3 p, n;
    int prim;
    int type;
    int degenerated;
} pvx;

typedef struct {
    int has_sv, has_direct;
    pvx sv, direct;
} subvx;

typedef struct {
    const lmo_accel* accel;
    const float* tris;
    const int32_t* tri_prim;
    size_t ntri;
    const lmo_pt_prim* prims;
    int nprims;
    /* lights: primitive ids, per-light triangle list + CDF, inverse area */
    int nlights;
    int* light_prims;
    int** light_tris;
    float** light_cdf;
    int* light_ntris;
    float* light_inv_area;
    int* prim_light; /* prim -> light index or -1 */
    /* sensor */
    v3 eye, vx, vy, vz;
    float tan_fov, aspect;
    int W, H;
    int max_v;
    int independent_light_dir;
    int ptmis;     /* 1: renderer::ptmis, 2: renderer::ptdirect, 3: renderer::ltdirect */
    int mis;       /* renderer::bdpt's weight: 0 misweight::powerheuristics, 1 misweight::simple */
    uint64_t num_samples, seed;
    int threads;
    double *sum, *sumsq;
    pthread_mutex_t lock;
} bd_job;

/* ---------------- surface interactions --------------------------------- */

static int bsdf_type(const lmo_pt_prim* P)
{
    switch (P->bsdf) {
    case LMO_BSDF_DIFFUSE: return T_D;
    case LMO_BSDF_DIELECTRIC: return T_S;
    case LMO_BSDF_COOK_TORRANCE: return T_G;
    default: return 0;
    }
}

static void basis(v3 a, v3* b, v3* c)
{
    *c = fabsf(a.x) > fabsf(a.y) ? normalize(V(a.z, 0.0f, -a.x)) : normalize(V(0.0f, a.z, -a.y));
    *b = cross(*c, a);
}
static v3 to_local(v3 n, v3 w)
{
    v3 b, c;
    basis(n, &b, &c);
    return V(dot(w, b), dot(w, c), dot(w, n));
}
static v3 to_world(v3 n, v3 l)
{
    v3 b, c;
    basis(n, &b, &c);
    return add(add(mul(b, l.x), mul(c, l.y)), mul(n, l.z));
}

static v3 cosine_hemisphere(float u0, float u1)
{
    float vx = 2.0f * u0 - 1.0f, vy = 2.0f * u1 - 1.0f, sx = 0.0f, sy = 0.0f;
    if (!(vx == 0.0f && vy == 0.0f)) {
        float r, th;
        if (vx > -vy) {
            if (vx > vy) { r = vx; th = (PI_F * 0.25f) * vy / vx; }
            else { r = vy; th = (PI_F * 0.25f) * (2.0f - vx / vy); }
        } else {
            if (vx < vy) { r = -vx; th = (PI_F * 0.25f) * (4.0f + vy / vx); }
            else { r = -vy; th = (PI_F * 0.25f) * (6.0f - vx / vy); }
        }
        sx = r * cosf(th);
        sy = r * sinf(th);
    }
    float z2 = 1.0f - sx * sx - sy * sy;
    return V(sx, sy, sqrtf(z2 > 0.0f ? z2 : 0.0f));
}

static float fresnel_dielectric(float wiDotN, float etaI, float etaT)
{
    const float eta = etaI / etaT;
    const float ct2 = 1.0f - eta * eta * (1.0f - wiDotN * wiDotN);
    if (ct2 <= 0.0f) return 1.0f;
    const float ci = fabsf(wiDotN), ct = sqrtf(ct2);
    const float rs = (etaI * ci - etaT * ct) / (etaI * ci + etaT * ct);
    const float rt = (etaI * ct - etaT * ci) / (etaI * ct + etaT * ci);
    return (rs * rs + rt * rt) * 0.5f;
}
static float ggx_d(v3 H, float a)
{
    const float c = H.z;
    if (c <= 0.0f) return 0.0f;
    const float t = 1.0f - c * c;
    const float tanH = t <= 0.0f ? 0.0f : sqrtf(t) / c;
    const float q = a * a + tanH * tanH;
    return (a * a) / (PI_F * c * c * c * c * q * q);
}
static v3 ggx_sample(float ua, float ub, float a)
{
    const float eps = 1e-4f;
    const float u0 = (1.0f - eps) * ua + eps, u1 = (1.0f - 2.0f * eps) * ub + eps;
    const float den = sqrtf(1.0f - (1.0f - a * a) * u0);
    const float cosT = sqrtf(1.0f - u0) / den, sinT = a * (sqrtf(u0) / den);
    const float phi = PI_F * (2.0f * u1 - 1.0f);
    return V(sinT * cosf(phi), sinT * sinf(phi), cosT);
}
static float fresnel_conductor(float c, float eta, float k)
{
    const float tmp = (eta * eta + k * k) * (c * c);
    const float rParl2 = (tmp - (eta * (2.0f * c)) + 1.0f) / (tmp + (eta * (2.0f * c)) + 1.0f);
    const float tmpF = eta * eta + k * k;
    const float rPerp2 = (tmpF - (eta * (2.0f * c)) + c * c) / (tmpF + (eta * (2.0f * c)) + c * c);
    return (rParl2 + rPerp2) * 0.5f;
}

/* BSDFUtils::ShadingNormalCorrection (bsdfutils.h:55-66) with sn = gn */
static float snc(v3 n, v3 wi, v3 wo, int dir)
{
    const float wig = dot(wi, n), wog = dot(wo, n);
    if (wig * wig <= 0.0f || wog * wog <= 0.0f) return 0.0f;
    (void)dir;
    return 1.0f;
}

/* Sensor_Pinhole raster position / importance (sensor_pinhole.cpp:137-185) */
static int raster_pos(const bd_job* J, v3 wo, float* rx, float* ry)
{
    const float ex = dot(J->vx, wo), ey = dot(J->vy, wo), ez = dot(J->vz, wo);
    if (ez >= 0.0f) return 0;
    *rx = (-ex / ez / J->tan_fov / J->aspect + 1.0f) * 0.5f;
    *ry = (-ey / ez / J->tan_fov + 1.0f) * 0.5f;
    if (*rx < 0.0f || *rx > 1.0f || *ry < 0.0f || *ry > 1.0f) return 0;
    return 1;
}
static float importance(const bd_job* J, v3 wo)
{
    float rx, ry;
    if (!raster_pos(J, wo, &rx, &ry)) return 0.0f;
    const float cosT = -dot(J->vz, wo);
    const float ic = 1.0f / cosT;
    return ic * ic * ic / (J->tan_fov * J->tan_fov * J->aspect * 4.0f);
}

/* Primitive::EvaluateDirection dispatch (primitive.h:84-199) */
static spd eval_dir(const bd_job* J, const pvx* v, int type, v3 wi, v3 wo, int dir, int evalDelta)
{
    if (type & T_E) return S1(importance(J, wo));
    if (type & T_L) {
        const lmo_pt_prim* P = &J->prims[v->prim];
        if (dot(wo, v->n) <= 0.0f) return S1(0.0f);
        return S3(P->Le);
    }
    if (v->prim < 0) return S1(0.0f);
    const lmo_pt_prim* P = &J->prims[v->prim];
    const v3 lwi = to_local(v->n, wi), lwo = to_local(v->n, wo);
    switch (P->bsdf) {
    case LMO_BSDF_DIFFUSE:
        if (lwi.z <= 0.0f || lwo.z <= 0.0f) return S1(0.0f);
        return sscale(S3(P->R), (1.0f / PI_F) * snc(v->n, wi, wo, dir));
    case LMO_BSDF_DIELECTRIC: {
        if (evalDelta) return S1(0.0f);
        float etaI = P->eta1, etaT = P->eta2;
        if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
        const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
        if (lwi.z * lwo.z >= 0.0f) return sscale(S3(P->R), Fr * snc(v->n, wi, wo, dir));
        const float eta = etaI / etaT;
        const float rc = dir == DIR_EL ? eta : 1.0f;
        return sscale(S3(P->R), (1.0f - Fr) * snc(v->n, wi, wo, dir) * rc * rc);
    }
    case LMO_BSDF_COOK_TORRANCE: {
        if (lwi.z <= 0.0f || lwo.z <= 0.0f) return S1(0.0f);
        const v3 H = normalize(add(lwi, lwo));
        const float D = ggx_d(H, P->roughness);
        const float woH = fabsf(dot(lwo, H));
        const float G = fminf(1.0f, fminf(2.0f * H.z * lwo.z / woH, 2.0f * H.z * lwi.z / woH));
        spd r;
        for (int k = 0; k < 3; k++)
            r.c[k] = P->R[k] * D * G * fresnel_conductor(dot(lwi, H), P->ct_eta[k], P->ct_k[k]) / (4.0f * lwi.z) /
                     lwo.z * snc(v->n, wi, wo, dir);
        return r;
    }
    default:
        return S1(0.0f);
    }
}

/* EvaluateDirectionPDF (projected solid angle) */
static float pdf_dir(const bd_job* J, const pvx* v, int type, v3 wi, v3 wo, int evalDelta)
{
    if (type & T_E) return importance(J, wo);
    if (type & T_L) return dot(wo, v->n) <= 0.0f ? 0.0f : 1.0f / PI_F;
    if (v->prim < 0) return 0.0f;
    const lmo_pt_prim* P = &J->prims[v->prim];
    const v3 lwi = to_local(v->n, wi), lwo = to_local(v->n, wo);
    switch (P->bsdf) {
    case LMO_BSDF_DIFFUSE:
        if (lwi.z <= 0.0f || lwo.z <= 0.0f) return 0.0f;
        return 1.0f / PI_F;
    case LMO_BSDF_DIELECTRIC: {
        if (evalDelta) return 0.0f;
        float etaI = P->eta1, etaT = P->eta2;
        if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
        const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
        return lwi.z * lwo.z >= 0.0f ? Fr : 1.0f - Fr;
    }
    case LMO_BSDF_COOK_TORRANCE: {
        if (lwi.z <= 0.0f || lwo.z <= 0.0f) return 0.0f;
        const v3 H = normalize(add(lwi, lwo));
        return ggx_d(H, P->roughness) * H.z / (4.0f * dot(lwo, H)) / lwo.z;
    }
    default:
        return 0.0f;
    }
}

static int is_delta_dir(const bd_job* J, const pvx* v, int type)
{
    if (type & (T_E | T_L)) return 0;
    return v->prim >= 0 && J->prims[v->prim].bsdf == LMO_BSDF_DIELECTRIC;
}
static int is_delta_pos(int type) { return (type & T_E) ? 1 : 0; }

/* EvaluatePositionGivenDirectionPDF / GivenPreviousPositionPDF (area measure) */
static float pdf_pos(const bd_job* J, const pvx* v)
{
    if (v->type & T_E || v->prim < 0) return 1.0f;
    return J->light_inv_area[J->prim_light[v->prim]];
}
static float emitter_pdf(const bd_job* J, const pvx* v)
{
    if (v->prim < 0) return 1.0f;
    return 1.0f / (float)J->nlights;
}

/* RenderUtils::GeometryTerm */
static float geometry_term(const pvx* a, const pvx* b)
{
    v3 d = sub(b->p, a->p);
    const float l2 = dot(d, d), l = sqrtf(l2);
    d = mul(d, 1.0f / l);
    float t = 1.0f;
    if (!a->degenerated) t *= fabsf(dot(a->n, d));
    if (!b->degenerated) t *= fabsf(dot(b->n, mul(d, -1.0f)));
    return t / l2;
}

/* Sample a light (uniform primitive, area-weighted triangle, uniform point) */
static int sample_light_pos(const bd_job* J, float u_sel, float ux, float uy, pvx* v, v3* tri_n)
{
    int li = (int)(u_sel * (float)J->nlights);
    li = li < 0 ? 0 : (li > J->nlights - 1 ? J->nlights - 1 : li);
    const float* cdf = J->light_cdf[li];
    const int nt = J->light_ntris[li];
    int lo = 0, hi = nt + 1; /* upper_bound over cdf[0..nt] */
    while (lo < hi) { const int m = (lo + hi) / 2; if (cdf[m] <= ux) lo = m + 1; else hi = m; }
    int i = lo - 1;
    i = i < 0 ? 0 : (i > nt - 1 ? nt - 1 : i);
    const float u2x = (ux - cdf[i]) / (cdf[i + 1] - cdf[i]);
    const float s = sqrtf(u2x > 0.0f ? u2x : 0.0f);
    const float bx = 1.0f - s, by = uy * s;
    const float* T = J->tris + 9 * (size_t)J->light_tris[li][i];
    const v3 p1 = V(T[0], T[1], T[2]), p2 = V(T[3], T[4], T[5]), p3 = V(T[6], T[7], T[8]);
    v->p = add(add(mul(p1, 1.0f - bx - by), mul(p2, bx)), mul(p3, by));
    v->n = normalize(cross(sub(p2, p1), sub(p3, p1)));
    v->prim = J->light_prims[li];
    v->degenerated = 0;
    if (tri_n) *tri_n = v->n;
    return 1;
}

static int trace(const bd_job* J, v3 o, v3 d, pvx* v)
{
    float r[8] = {o.x, o.y, o.z, EPS_ISECT, d.x, d.y, d.z, FLT_MAX};
    lmo_hit h;
    lmo_accel_trace(J->accel, r, 1, &h, 1);
    if (h.id < 0) return 0;
    const float* T = J->tris + 9 * (size_t)h.id;
    const v3 p1 = V(T[0], T[1], T[2]), p2 = V(T[3], T[4], T[5]), p3 = V(T[6], T[7], T[8]);
    v->p = V(h.p[0], h.p[1], h.p[2]);
    v->n = normalize(cross(sub(p2, p1), sub(p3, p1)));
    v->prim = J->tri_prim[h.id];
    v->type = bsdf_type(&J->prims[v->prim]);
    v->degenerated = 0;
    return 1;
}

static int visible(const bd_job* J, v3 a, v3 b)
{
    v3 d = sub(b, a);
    const float L = sqrtf(dot(d, d));
    d = mul(d, 1.0f / L);
    float r[8] = {a.x, a.y, a.z, EPS_ISECT, d.x, d.y, d.z, L * (1.0f - EPS_ISECT)};
    lmo_hit h;
    lmo_accel_trace(J->accel, r, 1, &h, 1);
    return h.id < 0;
}

/* BSDF SampleDirection; returns 0 where the reference leaves wo unset */
static int sample_dir(const bd_job* J, const pvx* v, v3 wi, float u0, float u1, float uc, v3* wo)
{
    if (v->prim < 0) return 0;
    const lmo_pt_prim* P = &J->prims[v->prim];
    const v3 lwi = to_local(v->n, wi);
    v3 lwo;
    switch (P->bsdf) {
    case LMO_BSDF_DIFFUSE:
        if (lwi.z <= 0.0f) return 0;
        lwo = cosine_hemisphere(u0, u1);
        break;
    case LMO_BSDF_DIELECTRIC: {
        float etaI = P->eta1, etaT = P->eta2;
        if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
        const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
        if (uc <= Fr) lwo = V(-lwi.x, -lwi.y, lwi.z);
        else {
            const float eta = etaI / etaT;
            const float ct2 = 1.0f - eta * eta * (1.0f - lwi.z * lwi.z);
            lwo = V(-eta * lwi.x, -eta * lwi.y, sqrtf(ct2 > 0.0f ? ct2 : 0.0f) * (lwi.z > 0.0f ? -1.0f : 1.0f));
        }
        break;
    }
    case LMO_BSDF_COOK_TORRANCE: {
        if (lwi.z <= 0.0f) return 0;
        const v3 H = ggx_sample(u0, u1, P->roughness);
        lwo = sub(mul(lwi, -1.0f), mul(H, 2.0f * dot(mul(lwi, -1.0f), H)));
        if (lwo.z <= 0.0f) return 0;
        break;
    }
    default:
        return 0;
    }
    *wo = to_world(v->n, lwo);
    return 1;
}

/* Subpath::Sample (renderer_bdpt.cpp:80-220) */
static int sample_subpath(const bd_job* J, uint64_t* rng, int dir, subvx* out)
{
    int n = 0;
    v3 initWo = zero3();
    for (int step = 0; J->max_v == -1 || step < J->max_v; step++) {
        if (step == 0) {
            pvx v;
            memset(&v, 0, sizeof(v));
            const float us = rnd(rng), a0 = rnd(rng), a1 = rnd(rng), b0 = rnd(rng), b1 = rnd(rng);
            if (dir == DIR_LE) {
                sample_light_pos(J, us, a0, a1, &v, NULL);
                v.type = T_L;
                /* direction from the same 2D sample as the position (light_area.cpp:73-80),
                 * or from its own sample for the diagnostic variant */
                initWo = J->independent_light_dir ? to_world(v.n, cosine_hemisphere(b0, b1))
                                                  : to_world(v.n, cosine_hemisphere(a0, a1));
            } else {
                v.p = J->eye;
                v.n = J->vz;
                v.prim = -1;
                v.type = T_E;
                v.degenerated = 1;
                const float rx = 2.0f * a0 - 1.0f, ry = 2.0f * a1 - 1.0f;
                const v3 we = normalize(V(J->aspect * J->tan_fov * rx, J->tan_fov * ry, -1.0f));
                initWo = add(add(mul(J->vx, we.x), mul(J->vy, we.y)), mul(J->vz, we.z));
            }
            memset(&out[n], 0, sizeof(subvx));
            out[n].has_sv = 1;
            out[n].sv = v;
            n++;
            continue;
        }
        const pvx* pv = &out[n - 1].sv;
        const pvx* ppv = n > 1 ? &out[n - 2].sv : NULL;
        subvx nv;
        memset(&nv, 0, sizeof(nv));
        /* BSDF-sampled vertex */
        {
            const v3 wi = ppv ? normalize(sub(ppv->p, pv->p)) : zero3();
            const float u0 = rnd(rng), u1 = rnd(rng), uc = rnd(rng);
            v3 wo = zero3();
            int ok = 1;
            if (step == 1) wo = initWo;
            else ok = sample_dir(J, pv, wi, u0, u1, uc, &wo);
            if (ok) {
                const spd f = eval_dir(J, pv, pv->type, wi, wo, dir, 0);
                if (!sblack(f) && trace(J, pv->p, wo, &nv.sv)) nv.has_sv = 1;
            }
        }
        /* direct vertex: the other end's emitter sampled from pv */
        {
            const float us = rnd(rng), a0 = rnd(rng), a1 = rnd(rng);
            pvx v;
            memset(&v, 0, sizeof(v));
            if (dir == DIR_LE) {
                v.p = J->eye;
                v.n = J->vz;
                v.prim = -1;
                v.type = T_E;
                v.degenerated = 1;
            } else {
                sample_light_pos(J, us, a0, a1, &v, NULL);
                v.type = T_L;
            }
            if (visible(J, pv->p, v.p)) {
                nv.has_direct = 1;
                nv.direct = v;
            }
        }
        if (nv.has_sv || nv.has_direct) out[n++] = nv;
        if (!nv.has_sv) break;
        if (rnd(rng) > 0.5f) break;
    }
    return n;
}

/* Path::Connect (renderer_bdpt.cpp:233-333) */
static int connect(const bd_job* J, int s, int t, int direct, const subvx* L, const subvx* E, pvx* path)
{
    int n = 0;
    if (s == 0 && t > 0) {
        if (!direct) {
            if (!E[t - 1].has_sv) return 0;
            if (E[t - 1].sv.prim < 0 || !J->prims[E[t - 1].sv.prim].is_light) return 0;
            for (int i = t - 1; i >= 0; i--) path[n++] = E[i].sv;
        } else {
            if (!E[t - 1].has_direct) return 0;
            path[n++] = E[t - 1].direct;
            for (int i = t - 2; i >= 0; i--) path[n++] = E[i].sv;
        }
        path[0].type = T_L;
    } else if (s > 0 && t == 0) {
        if (!direct) {
            /* a light subpath vertex is never the pinhole sensor */
            return 0;
        }
        if (!L[s - 1].has_direct) return 0;
        for (int i = 0; i < s - 1; i++) path[n++] = L[i].sv;
        path[n++] = L[s - 1].direct;
        path[n - 1].type = T_E;
    } else {
        if (!L[s - 1].has_sv || !E[t - 1].has_sv) return 0;
        if (!visible(J, L[s - 1].sv.p, E[t - 1].sv.p)) return 0;
        for (int i = 0; i < s; i++) path[n++] = L[i].sv;
        for (int i = t - 1; i >= 0; i--) path[n++] = E[i].sv;
    }
    return n;
}

static v3 dirto(const pvx* a, const pvx* b) { return normalize(sub(b->p, a->p)); }

/* EvaluateCst (renderer_bdpt.cpp:375-406) */
static spd eval_cst(const bd_job* J, const pvx* P, int n, int s)
{
    const int t = n - s;
    if (s == 0 && t > 0) {
        const pvx* v = &P[0];
        return sscale(eval_dir(J, v, v->type, zero3(), dirto(v, &P[1]), DIR_EL, 0), v->type & T_E ? 0.0f : 1.0f);
    }
    if (s > 0 && t == 0) {
        const pvx* v = &P[n - 1];
        /* EvaluatePosition(geom, true) of the pinhole is 0 */
        return sscale(eval_dir(J, v, v->type, zero3(), dirto(v, &P[n - 2]), DIR_LE, 0), 0.0f);
    }
    const pvx *vL = &P[s - 1], *vE = &P[s];
    const pvx* vLp = s - 2 >= 0 ? &P[s - 2] : NULL;
    const pvx* vEn = s + 1 < n ? &P[s + 1] : NULL;
    const spd fsL = eval_dir(J, vL, vL->type, vLp ? dirto(vL, vLp) : zero3(), dirto(vL, vE), DIR_LE, 1);
    const spd fsE = eval_dir(J, vE, vE->type, vEn ? dirto(vE, vEn) : zero3(), dirto(vE, vL), DIR_EL, 1);
    return sscale(smul(fsL, fsE), geometry_term(vL, vE));
}

/* EvaluateUnweightContribution (renderer_bdpt.cpp:489-591) */
static spd eval_unweighted(const bd_job* J, const pvx* P, int n, int s, int direct)
{
    const int t = n - s;
    spd aL = S1(1.0f);
    if (s > 0) {
        /* EvaluatePosition = 1 for area lights */
        aL = S1(1.0f / pdf_pos(J, &P[0]) / emitter_pdf(J, &P[0]));
        for (int i = 0; i < s - 1; i++) {
            const pvx *v = &P[i], *vn = &P[i + 1];
            const pvx* vp = i >= 1 ? &P[i - 1] : NULL;
            const v3 wi = vp ? dirto(v, vp) : zero3(), wo = dirto(v, vn);
            const int dl = t == 0 && i == s - 2 && direct;
            const spd fs = eval_dir(J, v, v->type, wi, wo, DIR_LE, dl);
            if (sblack(fs)) return S1(0.0f);
            const float pdf = dl ? pdf_pos(J, vn) / geometry_term(vn, v) * emitter_pdf(J, vn)
                                 : pdf_dir(J, v, v->type, wi, wo, 0);
            aL = smul(aL, sscale(fs, 1.0f / pdf));
        }
    }
    if (sblack(aL)) return S1(0.0f);
    spd aE = S1(1.0f);
    if (t > 0) {
        const pvx* v0 = &P[n - 1];
        /* sensor: EvaluatePosition 1, position pdf 1, emitter pdf 1 */
        aE = S1(1.0f / pdf_pos(J, v0) / emitter_pdf(J, v0));
        for (int i = n - 1; i > s; i--) {
            const pvx *v = &P[i], *vp = &P[i - 1];
            const pvx* vn = i < n - 1 ? &P[i + 1] : NULL;
            const v3 wi = vn ? dirto(v, vn) : zero3(), wo = dirto(v, vp);
            const int dl = s == 0 && i == 1 && direct;
            const spd fs = eval_dir(J, v, v->type, wi, wo, DIR_EL, dl);
            if (sblack(fs)) return S1(0.0f);
            const float pdf = dl ? pdf_pos(J, vp) / geometry_term(vp, v) * emitter_pdf(J, vp)
                                 : pdf_dir(J, v, v->type, wi, wo, 0);
            aE = smul(aE, sscale(fs, 1.0f / pdf));
        }
    }
    if (sblack(aE)) return S1(0.0f);
    const spd cst = eval_cst(J, P, n, s);
    if (sblack(cst)) return S1(0.0f);
    return smul(smul(aL, cst), aE);
}

/* Samplable + EvaluatePDF (renderer_bdpt.cpp:593-703) */
static float eval_pdf(const bd_job* J, const pvx* P, int n, int s, int direct)
{
    const int t = n - s;
    if (s > 0 && t > 0 && direct) return 0.0f;
    if (t == 0 && s > 0 && direct && is_delta_dir(J, &P[n - 2], P[n - 2].type)) return 0.0f;
    if (s == 0 && t > 0 && direct && is_delta_dir(J, &P[1], P[1].type)) return 0.0f;
    if (s == 0 && t > 0) {
        if (is_delta_pos(P[0].type)) return 0.0f;
    } else if (s > 0 && t == 0) {
        if (is_delta_pos(P[n - 1].type)) return 0.0f;
    } else {
        if (is_delta_dir(J, &P[s - 1], P[s - 1].type) || is_delta_dir(J, &P[s], P[s].type)) return 0.0f;
    }
    float pdf = 1.0f;
    if (s > 0) {
        pdf *= pdf_pos(J, &P[0]) * emitter_pdf(J, &P[0]);
        for (int i = 0; i < s - 1; i++) {
            const pvx *vi = &P[i], *vn = &P[i + 1];
            const pvx* vp = i >= 1 ? &P[i - 1] : NULL;
            if (t == 0 && i == s - 2 && direct) pdf *= pdf_pos(J, vn) * emitter_pdf(J, vn);
            else pdf *= pdf_dir(J, vi, vi->type, vp ? dirto(vi, vp) : zero3(), dirto(vi, vn), 0) * geometry_term(vi, vn);
        }
    }
    if (t > 0) {
        pdf *= pdf_pos(J, &P[n - 1]) * emitter_pdf(J, &P[n - 1]);
        for (int i = n - 1; i >= s + 1; i--) {
            const pvx *vi = &P[i], *vp = &P[i - 1];
            const pvx* vn = i + 1 < n ? &P[i + 1] : NULL;
            if (s == 0 && i == s + 1 && direct) pdf *= pdf_pos(J, vp) * emitter_pdf(J, vp);
            else pdf *= pdf_dir(J, vi, vi->type, vn ? dirto(vi, vn) : zero3(), dirto(vi, vp), 0) * geometry_term(vi, vp);
        }
    }
    return pdf;
}

/* MISWeight_Simple (renderer_bdpt.cpp:711-744): one over the number of
 * strategies that can sample the path */
static float mis_simple(const bd_job* J, const pvx* P, int n)
{
    int nonzero = 0;
    for (int s = 0; s <= n; s++)
        for (int d = 0; d < 2; d++) {
            const int t = n - s;
            if (s > 0 && t > 0 && d) continue;
            if (eval_pdf(J, P, n, s, d) > 0.0f) nonzero++;
        }
    return 1.0f / (float)nonzero;
}

/* MISWeight_PowerHeuristics (renderer_bdpt.cpp:747-784) */
static float mis_power(const bd_job* J, const pvx* P, int n, int s_, int d_)
{
    if (J->mis == 1) return mis_simple(J, P, n);
    const float ps = eval_pdf(J, P, n, s_, d_);
    float inv = 0.0f;
    for (int s = 0; s <= n; s++)
        for (int d = 0; d < 2; d++) {
            const int t = n - s;
            if (s > 0 && t > 0 && d) continue;
            const float pi = eval_pdf(J, P, n, s, d);
            if (pi > 0.0f) {
                const float r = pi / ps;
                inv += r * r;
            }
        }
    return 1.0f / inv;
}

#define MAXV 64

static void* bd_worker(void* arg)
{
    void** a = (void**)arg;
    bd_job* J = (bd_job*)a[0];
    const int wi_ = (int)(intptr_t)a[1];
    const int W = J->W, H = J->H;
    double* sum = (double*)calloc((size_t)W * H * 3, sizeof(double));
    double* sumsq = (double*)calloc((size_t)W * H * 3, sizeof(double));
    uint64_t rng = J->seed ^ 0x6A09E667F3BCC909ull;
    rng = splitmix64(&rng) ^ ((uint64_t)wi_ * 0xA0761D6478BD642Full);
    rng = splitmix64(&rng);
    subvx L[MAXV], E[MAXV];
    pvx path[2 * MAXV];
    int pix_list[4 * MAXV * MAXV];
    double val_list[4 * MAXV * MAXV][3];
    const uint64_t b = J->num_samples * (uint64_t)wi_ / (uint64_t)J->threads;
    const uint64_t e = J->num_samples * (uint64_t)(wi_ + 1) / (uint64_t)J->threads;
    for (uint64_t smp = b; smp < e; smp++) {
        const int nL = sample_subpath(J, &rng, DIR_LE, L);
        const int nE = sample_subpath(J, &rng, DIR_EL, E);
        int nsplat = 0;
        for (int n = 2; n <= nE + nL; n++) {
            if (J->max_v != -1 && n > J->max_v) continue;
            const int minS = n - nE > 0 ? n - nE : 0;
            const int maxS = nL < n ? nL : n;
            for (int s = minS; s <= maxS; s++)
                for (int d = 0; d < 2; d++) {
                    const int t = n - s;
                    if (s > 0 && t > 0 && d) continue;
                    const int np = connect(J, s, t, d, L, E, path);
                    if (!np) continue;
                    const spd cs = eval_unweighted(J, path, np, s, d);
                    if (sblack(cs)) continue;
                    const float w = mis_power(J, path, np, s, d);
                    /* SelectionPDF: 0.5 per roulette step survived */
                    float sel = 1.0f;
                    for (int i = 1; i < s - 1; i++) sel *= 0.5f;
                    for (int i = 1; i < t - 1; i++) sel *= 0.5f;
                    const spd C = sscale(cs, w / sel);
                    if (sblack(C) || !(w == w)) continue;
                    float rx = 0.0f, ry = 0.0f;
                    raster_pos(J, dirto(&path[np - 1], &path[np - 2]), &rx, &ry);
                    int ix = (int)(rx * (float)W), iy = (int)(ry * (float)H);
                    ix = ix < 0 ? 0 : (ix > W - 1 ? W - 1 : ix);
                    iy = iy < 0 ? 0 : (iy > H - 1 ? H - 1 : iy);
                    const int pix = iy * W + ix;
                    int k;
                    for (k = 0; k < nsplat; k++)
                        if (pix_list[k] == pix) break;
                    if (k == nsplat) {
                        pix_list[nsplat] = pix;
                        val_list[nsplat][0] = val_list[nsplat][1] = val_list[nsplat][2] = 0.0;
                        nsplat++;
                    }
                    for (int c = 0; c < 3; c++) val_list[k][c] += C.c[c];
                }
        }
        for (int k = 0; k < nsplat; k++)
            for (int c = 0; c < 3; c++) {
                sum[3 * (size_t)pix_list[k] + c] += val_list[k][c];
                sumsq[3 * (size_t)pix_list[k] + c] += val_list[k][c] * val_list[k][c];
            }
    }
    pthread_mutex_lock(&J->lock);
    for (size_t i = 0; i < (size_t)W * H * 3; i++) { J->sum[i] += sum[i]; J->sumsq[i] += sumsq[i]; }
    pthread_mutex_unlock(&J->lock);
    free(sum);
    free(sumsq);
    return NULL;
}

/* Splat accumulation of one sample: contributions merged per pixel before
 * their squares are summed, as the reference film does per sample. */
typedef struct {
    int n;
    int pix[4 * MAXV];
    double val[4 * MAXV][3];
} splat_list;

static void splat_add(splat_list* L, int pix, spd C)
{
    int k;
    for (k = 0; k < L->n; k++)
        if (L->pix[k] == pix) break;
    if (k == L->n) {
        if (L->n == 4 * MAXV) return;
        L->pix[k] = pix;
        L->val[k][0] = L->val[k][1] = L->val[k][2] = 0.0;
        L->n++;
    }
    for (int c = 0; c < 3; c++) L->val[k][c] += C.c[c];
}

static int pixel_of(const bd_job* J, float rx, float ry)
{
    int ix = (int)(rx * (float)J->W), iy = (int)(ry * (float)J->H);
    ix = ix < 0 ? 0 : (ix > J->W - 1 ? J->W - 1 : ix);
    iy = iy < 0 ? 0 : (iy > J->H - 1 ? J->H - 1 : iy);
    return iy * J->W + ix;
}

/* Renderer_PTMIS sample closure (renderer_ptmis.cpp:80-305); with
 * J->ptmis == 2 the Renderer_PTDirect one (renderer_ptdirect.cpp:84-276). */
static void* ptmis_worker(void* arg)
{
    void** a = (void**)arg;
    bd_job* J = (bd_job*)a[0];
    const int wi_ = (int)(intptr_t)a[1];
    const int W = J->W, H = J->H;
    double* sum = (double*)calloc((size_t)W * H * 3, sizeof(double));
    double* sumsq = (double*)calloc((size_t)W * H * 3, sizeof(double));
    uint64_t rng = J->seed ^ 0x3C6EF372FE94F82Bull;
    rng = splitmix64(&rng) ^ ((uint64_t)wi_ * 0xA0761D6478BD642Full);
    rng = splitmix64(&rng);
    splat_list* sl = (splat_list*)malloc(sizeof(splat_list));
    const float pdfL = 1.0f / (float)J->nlights;
    const uint64_t b = J->num_samples * (uint64_t)wi_ / (uint64_t)J->threads;
    const uint64_t e = J->num_samples * (uint64_t)(wi_ + 1) / (uint64_t)J->threads;
    for (uint64_t smp = b; smp < e; smp++) {
        sl->n = 0;
        /* sensor: uniform raster position over the film (sensor_pinhole.cpp:79-90) */
        pvx cur;
        cur.p = J->eye;
        cur.n = J->vz;
        cur.prim = -1;
        cur.type = T_E;
        cur.degenerated = 1;
        const float r0 = 2.0f * rnd(&rng) - 1.0f, r1 = 2.0f * rnd(&rng) - 1.0f;
        const v3 we = normalize(V(J->aspect * J->tan_fov * r0, J->tan_fov * r1, -1.0f));
        const v3 initWo = add(add(mul(J->vx, we.x), mul(J->vy, we.y)), mul(J->vz, we.z));
        float rx0, ry0;
        if (!raster_pos(J, initWo, &rx0, &ry0)) continue;
        const int pix0 = pixel_of(J, rx0, ry0);
        spd thr = S1(1.0f);
        v3 wi = zero3();
        int nv = 1;
        for (;;) {
            if (J->max_v != -1 && nv >= J->max_v) break;
            /* direct light sampling (:131-193) */
            {
                const float us = rnd(&rng), u0 = rnd(&rng), u1 = rnd(&rng);
                pvx L;
                sample_light_pos(J, us, u0, u1, &L, NULL);
                L.type = T_L;
                const v3 ppL = normalize(sub(L.p, cur.p));
                const spd fsE = eval_dir(J, &cur, cur.type, wi, ppL, DIR_EL, 1);
                const spd fsL = eval_dir(J, &L, T_L, zero3(), mul(ppL, -1.0f), DIR_LE, 0);
                const float G = geometry_term(&cur, &L);
                const float pdfPL = J->light_inv_area[J->prim_light[L.prim]];
                spd C = smul(thr, smul(fsE, fsL));
                C = sscale(C, G / pdfL / pdfPL);
                if (!sblack(C) && visible(J, cur.p, L.p)) {
                    const float pdfDL = pdfPL / G * pdfL;
                    const float pdfB = pdf_dir(J, &cur, cur.type, wi, ppL, 1);
                    const float w = J->ptmis == 2 ? 1.0f : pdfDL / (pdfDL + pdfB);
                    int pix = pix0;
                    if (cur.type == T_E) {
                        float rx, ry;
                        if (raster_pos(J, ppL, &rx, &ry)) pix = pixel_of(J, rx, ry);
                    }
                    splat_add(sl, pix, sscale(C, w));
                }
            }
            /* next direction (:197-224) */
            v3 wo;
            if (cur.type == T_E) {
                wo = initWo;
            } else {
                const float u0 = rnd(&rng), u1 = rnd(&rng), uc = rnd(&rng);
                if (!sample_dir(J, &cur, wi, u0, u1, uc, &wo)) break;
            }
            const float pdfD = pdf_dir(J, &cur, cur.type, wi, wo, 0);
            const spd fs = eval_dir(J, &cur, cur.type, wi, wo, DIR_EL, 0);
            if (sblack(fs)) break;
            thr = smul(thr, sscale(fs, 1.0f / pdfD));
            pvx hit;
            if (!trace(J, cur.p, wo, &hit)) break;
            /* BSDF-sampled light hit (:240-273) */
            if (J->ptmis == 1 && J->prims[hit.prim].is_light) {
                const float pdfDL = (cur.type & T_S)
                                        ? 0.0f
                                        : J->light_inv_area[J->prim_light[hit.prim]] / geometry_term(&hit, &cur) * pdfL;
                const float w = pdfD / (pdfD + pdfDL);
                pvx hl = hit;
                hl.type = T_L;
                const spd Le = eval_dir(J, &hl, T_L, zero3(), mul(wo, -1.0f), DIR_EL, 0);
                const spd C = smul(thr, Le);
                if (!sblack(C)) splat_add(sl, pix0, sscale(C, w));
            }
            /* roulette (:285-293) */
            if (rnd(&rng) > 0.5f) break;
            thr = sscale(thr, 2.0f);
            cur = hit;
            wi = mul(wo, -1.0f);
            nv++;
        }
        for (int k = 0; k < sl->n; k++)
            for (int c = 0; c < 3; c++) {
                sum[3 * (size_t)sl->pix[k] + c] += sl->val[k][c];
                sumsq[3 * (size_t)sl->pix[k] + c] += sl->val[k][c] * sl->val[k][c];
            }
    }
    pthread_mutex_lock(&J->lock);
    for (size_t i = 0; i < (size_t)W * H * 3; i++) { J->sum[i] += sum[i]; J->sumsq[i] += sumsq[i]; }
    pthread_mutex_unlock(&J->lock);
    free(sl);
    free(sum);
    free(sumsq);
    return NULL;
}

/* Renderer_LTDirect sample closure (renderer_ltdirect.cpp:74-276): a light
 * path (light primitive uniformly, area-CDF triangle, uniform point, the
 * emission direction from the same 2D sample as the position,
 * light_area.cpp:73-80), connected to the sensor at every vertex with
 * weight 1 (:118-168), extended by BSDF sampling (:170-205), Russian roulette
 * 0.5 after each hit (:223-235).  Every splat lands where its connection
 * meets the film. */
static void* lt_worker(void* arg)
{
    void** a = (void**)arg;
    bd_job* J = (bd_job*)a[0];
    const int wi_ = (int)(intptr_t)a[1];
    const int W = J->W, H = J->H;
    double* sum = (double*)calloc((size_t)W * H * 3, sizeof(double));
    double* sumsq = (double*)calloc((size_t)W * H * 3, sizeof(double));
    uint64_t rng = J->seed ^ 0x510E527FADE682D1ull;
    rng = splitmix64(&rng) ^ ((uint64_t)wi_ * 0xA0761D6478BD642Full);
    rng = splitmix64(&rng);
    splat_list* sl = (splat_list*)malloc(sizeof(splat_list));
    const float pdfL = 1.0f / (float)J->nlights;
    const uint64_t b = J->num_samples * (uint64_t)wi_ / (uint64_t)J->threads;
    const uint64_t e = J->num_samples * (uint64_t)(wi_ + 1) / (uint64_t)J->threads;
    pvx E;
    E.p = J->eye;
    E.n = J->vz;
    E.prim = -1;
    E.type = T_E;
    E.degenerated = 1;
    for (uint64_t smp = b; smp < e; smp++) {
        sl->n = 0;
        pvx cur;
        const float us = rnd(&rng), a0 = rnd(&rng), a1 = rnd(&rng);
        sample_light_pos(J, us, a0, a1, &cur, NULL);
        cur.type = T_L;
        /* the reference draws the emission direction from the position's 2D
         * sample; the diagnostic variant draws a fresh one */
        float d0 = a0, d1 = a1;
        if (J->independent_light_dir) { d0 = rnd(&rng); d1 = rnd(&rng); }
        const v3 initWo = to_world(cur.n, cosine_hemisphere(d0, d1));
        const float pdfPL = J->light_inv_area[J->prim_light[cur.prim]];
        spd thr = S1(1.0f / pdfPL / pdfL);
        v3 wi = zero3();
        int nv = 1;
        for (;;) {
            if (J->max_v != -1 && nv >= J->max_v) break;
            /* sensor connection (:118-168); pdf_E = pdf_PE = We_P = 1 for the pinhole */
            {
                const v3 ppE = normalize(sub(E.p, cur.p));
                const spd fsL = eval_dir(J, &cur, cur.type, wi, ppE, DIR_LE, 1);
                const spd fsE = eval_dir(J, &E, T_E, zero3(), mul(ppE, -1.0f), DIR_EL, 0);
                const float G = geometry_term(&cur, &E);
                const spd C = sscale(smul(thr, smul(fsL, fsE)), G);
                float rx, ry;
                if (!sblack(C) && raster_pos(J, mul(ppE, -1.0f), &rx, &ry) && visible(J, cur.p, E.p))
                    splat_add(sl, pixel_of(J, rx, ry), C);
            }
            /* next direction (:170-205) */
            v3 wo;
            if (cur.type == T_L) {
                wo = initWo;
            } else {
                const float u0 = rnd(&rng), u1 = rnd(&rng), uc = rnd(&rng);
                if (!sample_dir(J, &cur, wi, u0, u1, uc, &wo)) break;
            }
            const float pdfD = pdf_dir(J, &cur, cur.type, wi, wo, 0);
            const spd fs = eval_dir(J, &cur, cur.type, wi, wo, DIR_LE, 0);
            if (sblack(fs)) break;
            thr = smul(thr, sscale(fs, 1.0f / pdfD));
            pvx hit;
            if (!trace(J, cur.p, wo, &hit)) break;
            /* roulette (:223-235) */
            if (rnd(&rng) > 0.5f) break;
            thr = sscale(thr, 2.0f);
            cur = hit;
            wi = mul(wo, -1.0f);
            nv++;
        }
        for (int k = 0; k < sl->n; k++)
            for (int c = 0; c < 3; c++) {
                sum[3 * (size_t)sl->pix[k] + c] += sl->val[k][c];
                sumsq[3 * (size_t)sl->pix[k] + c] += sl->val[k][c] * sl->val[k][c];
            }
    }
    pthread_mutex_lock(&J->lock);
    for (size_t i = 0; i < (size_t)W * H * 3; i++) { J->sum[i] += sum[i]; J->sumsq[i] += sumsq[i]; }
    pthread_mutex_unlock(&J->lock);
    free(sl);
    free(sum);
    free(sumsq);
    return NULL;
}

uint64_t lmo_render_bdpt(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims, int nprims,
                         const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices, uint64_t seed,
                         int threads, double* sum, double* sumsq)
{
    return lmo_render_bdpt_ex(tris, tri_prim, ntri, prims, nprims, cam, num_samples, max_num_vertices, seed, threads,
                              sum, sumsq, 0);
}

uint64_t lmo_render_ptmis(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims, int nprims,
                          const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices, uint64_t seed,
                          int threads, double* sum, double* sumsq)
{
    return lmo_render_bdpt_ex(tris, tri_prim, ntri, prims, nprims, cam, num_samples, max_num_vertices, seed, threads,
                              sum, sumsq, -1);
}

uint64_t lmo_render_ptdirect(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                             int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                             uint64_t seed, int threads, double* sum, double* sumsq)
{
    return lmo_render_bdpt_ex(tris, tri_prim, ntri, prims, nprims, cam, num_samples, max_num_vertices, seed, threads,
                              sum, sumsq, -2);
}

uint64_t lmo_render_ltdirect(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                             int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                             uint64_t seed, int threads, double* sum, double* sumsq)
{
    return lmo_render_bdpt_ex(tris, tri_prim, ntri, prims, nprims, cam, num_samples, max_num_vertices, seed, threads,
                              sum, sumsq, -3);
}

/* independent_light_dir: 0 / 1 select the BDPT variants; -1 runs
 * renderer::ptmis, -2 renderer::ptdirect, -3 renderer::ltdirect, -4
 * renderer::ltdirect with an independent emission-direction sample */
uint64_t lmo_render_bdpt_ex(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                            int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                            uint64_t seed, int threads, double* sum, double* sumsq, int independent_light_dir)
{
    return lmo_render_bdpt_mis(tris, tri_prim, ntri, prims, nprims, cam, num_samples, max_num_vertices, seed, threads,
                               sum, sumsq, independent_light_dir, 0);
}

/* Scene tables of a job: the oracle's accel::bvh_sahbin, per-light triangle
 * lists with their area CDFs and inverse areas, and the sensor basis
 * (scene3.cpp:213-221). */
static void bd_job_init(bd_job* J, const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                        int nprims, const lmo_pt_camera* cam)
{
    memset(J, 0, sizeof(*J));
    J->accel = lmo_accel_build(1, tris, ntri);
    J->tris = tris;
    J->tri_prim = tri_prim;
    J->ntri = ntri;
    J->prims = prims;
    J->nprims = nprims;
    J->prim_light = (int*)malloc(sizeof(int) * (size_t)nprims);
    for (int i = 0; i < nprims; i++) {
        J->prim_light[i] = -1;
        if (prims[i].is_light) J->prim_light[i] = J->nlights++;
    }
    J->light_prims = (int*)malloc(sizeof(int) * (size_t)(J->nlights + 1));
    J->light_tris = (int**)calloc((size_t)(J->nlights + 1), sizeof(int*));
    J->light_cdf = (float**)calloc((size_t)(J->nlights + 1), sizeof(float*));
    J->light_ntris = (int*)calloc((size_t)(J->nlights + 1), sizeof(int));
    J->light_inv_area = (float*)calloc((size_t)(J->nlights + 1), sizeof(float));
    for (int i = 0; i < nprims; i++) {
        const int li = J->prim_light[i];
        if (li < 0) continue;
        J->light_prims[li] = i;
        int cnt = 0;
        for (size_t k = 0; k < ntri; k++) cnt += tri_prim[k] == i;
        J->light_ntris[li] = cnt;
        J->light_tris[li] = (int*)malloc(sizeof(int) * (size_t)cnt);
        J->light_cdf[li] = (float*)malloc(sizeof(float) * (size_t)(cnt + 1));
        float sa = 0.0f;
        int j = 0;
        J->light_cdf[li][0] = 0.0f;
        for (size_t k = 0; k < ntri; k++) {
            if (tri_prim[k] != i) continue;
            const float* T = tris + 9 * k;
            const v3 p1 = V(T[0], T[1], T[2]), p2 = V(T[3], T[4], T[5]), p3 = V(T[6], T[7], T[8]);
            const v3 c = cross(sub(p2, p1), sub(p3, p1));
            const float area = sqrtf(dot(c, c)) * 0.5f;
            J->light_tris[li][j] = (int)k;
            J->light_cdf[li][j + 1] = J->light_cdf[li][j] + area;
            sa += area;
            j++;
        }
        for (int q = 0; q <= cnt; q++) J->light_cdf[li][q] /= J->light_cdf[li][cnt];
        J->light_inv_area[li] = 1.0f / sa;
    }
    J->eye = V(cam->eye[0], cam->eye[1], cam->eye[2]);
    const v3 c = V(cam->center[0], cam->center[1], cam->center[2]);
    const v3 up = V(cam->up[0], cam->up[1], cam->up[2]);
    J->vz = normalize(sub(J->eye, c));
    J->vx = normalize(cross(up, J->vz));
    J->vy = cross(J->vz, J->vx);
    J->tan_fov = tanf(cam->fov_deg * PI_F / 180.0f * 0.5f);
    J->aspect = (float)cam->width / (float)cam->height;
    J->W = cam->width;
    J->H = cam->height;
}

static void bd_job_release(bd_job* J)
{
    for (int li = 0; li < J->nlights; li++) { free(J->light_tris[li]); free(J->light_cdf[li]); }
    free(J->light_prims); free(J->light_tris); free(J->light_cdf); free(J->light_ntris); free(J->light_inv_area);
    free(J->prim_light);
    lmo_accel_free((lmo_accel*)J->accel);
}

/* Runs fn on J->threads workers, each given (J, worker index). */
static void bd_run_workers(bd_job* J, void* (*fn)(void*), void* ctx)
{
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)J->threads);
    void** args = (void**)malloc(sizeof(void*) * 3 * (size_t)J->threads);
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, (size_t)64 << 20);
    for (int i = 0; i < J->threads; i++) {
        args[3 * i] = J;
        args[3 * i + 1] = (void*)(intptr_t)i;
        args[3 * i + 2] = ctx;
        pthread_create(&th[i], &attr, fn, &args[3 * i]);
    }
    for (int i = 0; i < J->threads; i++) pthread_join(th[i], NULL);
    pthread_attr_destroy(&attr);
    free(th);
    free(args);
}

uint64_t lmo_render_bdpt_mis(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                             int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                             uint64_t seed, int threads, double* sum, double* sumsq, int independent_light_dir,
                             int mis)
{
    bd_job J;
    bd_job_init(&J, tris, tri_prim, ntri, prims, nprims, cam);
    J.mis = mis;
    if (max_num_vertices > MAXV || max_num_vertices == -1) max_num_vertices = MAXV;
    J.max_v = max_num_vertices;
    J.independent_light_dir = independent_light_dir > 0 || independent_light_dir == -4;
    J.ptmis = independent_light_dir == -4 ? 3 : (independent_light_dir < 0 ? -independent_light_dir : 0);
    J.num_samples = num_samples;
    J.seed = seed;
    J.threads = threads < 1 ? 1 : threads;
    J.sum = sum;
    J.sumsq = sumsq;
    memset(sum, 0, sizeof(double) * (size_t)J.W * J.H * 3);
    memset(sumsq, 0, sizeof(double) * (size_t)J.W * J.H * 3);
    pthread_mutex_init(&J.lock, NULL);
    if (J.nlights > 0) bd_run_workers(&J, J.ptmis == 3 ? lt_worker : (J.ptmis ? ptmis_worker : bd_worker), NULL);
    pthread_mutex_destroy(&J.lock);
    bd_job_release(&J);
    return num_samples;
}

/* ======================= renderer::vcm ====================================
 * Restates src/liblightmetrica/renderer/renderer_vcm.cpp, the reference's
 * naive vertex connection and merging (Georgiev et al. 2012 in the path-space
 * form of Hachisuka et al. 2012):
 *   SubpathSampler::TraceSubpath  subpathsampler.cpp:41-190: no roulette; a
 *       subpath ends on a miss, on a black BSDF value or after
 *       max_num_vertices vertices; the emitter's position and direction both
 *       come from the direction sample uED (light_area.cpp:73-80)
 *   VCMPath::ConnectSubpaths  :73-100     MergeSubpaths  :102-113
 *   VCMPath::EvaluateF        :115-211    EvaluatePathPDF :213-276
 *   EvaluateMISWeight_VCM / _BDPT / _BDPM :278-338
 *   VCMKdTree::Build / RangeQuery :355-465: light subpath vertices 1.. that
 *       are neither a delta position nor a delta direction, |p - x|^2 < r^2
 *   Render :596-790: per pass the radius r = r0, then sqrt((alpha + k) /
 *       (1 + k)) r; num_photon_trace_samples light subpaths and their range
 *       structure; num_eye_trace_samples samples, each an eye subpath and a
 *       fresh light subpath: connections s in [max(0, 2 - t, min - t),
 *       min(nL, max - t)], merges at each eye vertex that is not a delta
 *       position; splats C W H / N_E; the film is the mean of the passes.
 * The range structure here is a grid of cells 2r wide (entries sorted by
 * cell), which returns the same vertex set as the kd-tree.  The reference's
 * "if (p.v == 0) return;" in the connection loop (:698-702) ends the whole
 * sample, and does so here too.  Random numbers: one stream per photon
 * subpath and per eye sample, keyed by (seed, pass, index). */

typedef struct {
    int mode; /* 0 vcm, 1 bdpt, 2 bdpm */
    int min_v;
    uint64_t n_photon, n_eye;
    float r, inv_cell;
    uint64_t pass;
    /* photon subpaths: vertex k of subpath i at pool_v[i * max_v + k] */
    pvx* pool_v;
    int* pool_n;
    /* range structure: eligible photon vertices sorted by cell key */
    int64_t* keys;
    int32_t* ent; /* subpath * 64 + vertex */
    size_t nent;
} vcm_ctx;

static uint64_t vcm_stream(uint64_t seed, uint64_t pass, uint64_t index, uint64_t kind)
{
    uint64_t s = seed ^ 0x9E3779B97F4A7C15ull;
    s = splitmix64(&s) ^ (pass * 0xD1B54A32D192ED03ull);
    s = splitmix64(&s) ^ (index * 0xA0761D6478BD642Full) ^ kind;
    return splitmix64(&s);
}

/* SubpathSampler::TraceSubpath (subpathsampler.cpp:41-190) */
static int vcm_subpath(const bd_job* J, uint64_t* rng, int dir, pvx* out)
{
    int n = 0;
    v3 initWo = zero3();
    for (int step = 0; step < J->max_v; step++) {
        if (step == 0) {
            /* uEP (2D), uEP_C, uED (2D), uED_C in this order (:67-76) */
            (void)rnd(rng);
            (void)rnd(rng);
            const float uc = rnd(rng), d0 = rnd(rng), d1 = rnd(rng);
            (void)rnd(rng);
            pvx v;
            memset(&v, 0, sizeof(v));
            if (dir == DIR_LE) {
                sample_light_pos(J, uc, d0, d1, &v, NULL);
                v.type = T_L;
                initWo = to_world(v.n, cosine_hemisphere(d0, d1));
            } else {
                v.p = J->eye;
                v.n = J->vz;
                v.prim = -1;
                v.type = T_E;
                v.degenerated = 1;
                const float rx = 2.0f * d0 - 1.0f, ry = 2.0f * d1 - 1.0f;
                const v3 we = normalize(V(J->aspect * J->tan_fov * rx, J->tan_fov * ry, -1.0f));
                initWo = add(add(mul(J->vx, we.x), mul(J->vy, we.y)), mul(J->vz, we.z));
            }
            out[n++] = v;
            continue;
        }
        const pvx* pv = &out[n - 1];
        v3 wi = zero3(), wo = zero3();
        if (step == 1) {
            wo = initWo;
        } else {
            wi = normalize(sub(out[n - 2].p, pv->p));
            const float u0 = rnd(rng), u1 = rnd(rng), uc = rnd(rng);
            if (!sample_dir(J, pv, wi, u0, u1, uc, &wo)) break; /* wo left zero: black below */
        }
        if (sblack(eval_dir(J, pv, pv->type, wi, wo, dir, 0))) break;
        pvx v;
        if (!trace(J, pv->p, wo, &v)) break;
        out[n++] = v;
    }
    return n;
}

/* VCMPath::EvaluateF (renderer_vcm.cpp:115-211).  EvaluatePosition is 1 for
 * the area lights and the pinhole without evalDelta; with it, 0 for the
 * pinhole (a delta position). */
static spd vcm_eval_f(const bd_job* J, const pvx* P, int n, int s, int merge)
{
    const int t = n - s;
    spd fL = S1(1.0f);
    if (s > 0) {
        const int m = merge ? s : s - 1;
        for (int i = 0; i < m; i++) {
            const v3 wi = i >= 1 ? dirto(&P[i], &P[i - 1]) : zero3();
            fL = smul(fL, eval_dir(J, &P[i], P[i].type, wi, dirto(&P[i], &P[i + 1]), DIR_LE, 0));
            fL = sscale(fL, geometry_term(&P[i], &P[i + 1]));
        }
    }
    if (sblack(fL)) return S1(0.0f);
    spd fE = S1(1.0f);
    if (t > 0) {
        for (int i = n - 1; i > s; i--) {
            const v3 wi = i < n - 1 ? dirto(&P[i], &P[i + 1]) : zero3();
            fE = smul(fE, eval_dir(J, &P[i], P[i].type, wi, dirto(&P[i], &P[i - 1]), DIR_EL, 0));
            fE = sscale(fE, geometry_term(&P[i], &P[i - 1]));
        }
    }
    if (sblack(fE)) return S1(0.0f);
    spd cst;
    if (!merge) {
        if (s == 0 && t > 0) {
            cst = sscale(eval_dir(J, &P[0], P[0].type, zero3(), dirto(&P[0], &P[1]), DIR_EL, 0),
                         (P[0].type & T_E) ? 0.0f : 1.0f);
        } else if (s > 0 && t == 0) {
            cst = S1(0.0f); /* the pinhole end: EvaluatePosition(evalDelta = true) = 0 */
        } else {
            const pvx *vL = &P[s - 1], *vE = &P[s];
            const spd fsL = eval_dir(J, vL, vL->type, s - 2 >= 0 ? dirto(vL, &P[s - 2]) : zero3(), dirto(vL, vE),
                                     DIR_LE, 1);
            const spd fsE = eval_dir(J, vE, vE->type, s + 1 < n ? dirto(vE, &P[s + 1]) : zero3(), dirto(vE, vL),
                                     DIR_EL, 1);
            cst = smul(sscale(fsL, geometry_term(vL, vE)), fsE);
        }
    } else {
        const pvx* v = &P[s];
        cst = eval_dir(J, v, v->type, dirto(v, &P[s + 1]), dirto(v, &P[s - 1]), DIR_EL, 1);
    }
    return smul(smul(fL, cst), fE);
}

/* VCMPath::EvaluatePathPDF (renderer_vcm.cpp:213-276), area product measure */
static float vcm_path_pdf(const bd_job* J, const pvx* P, int n, int s, int merge, float r)
{
    const int t = n - s;
    if (!merge) {
        if (s == 0 && t > 0) {
            if (is_delta_pos(P[0].type)) return 0.0f;
        } else if (s > 0 && t == 0) {
            if (is_delta_pos(P[n - 1].type)) return 0.0f;
        } else if (s > 0 && t > 0) {
            if (is_delta_dir(J, &P[s - 1], P[s - 1].type) || is_delta_dir(J, &P[s], P[s].type)) return 0.0f;
        }
    } else {
        if (s == 0 || t == 0) return 0.0f;
        if (is_delta_pos(P[s].type) || is_delta_dir(J, &P[s], P[s].type)) return 0.0f;
    }
    float pdf = 1.0f;
    if (s > 0) {
        pdf *= pdf_pos(J, &P[0]) * emitter_pdf(J, &P[0]);
        const int m = merge ? s : s - 1;
        for (int i = 0; i < m; i++) {
            const v3 wi = i >= 1 ? dirto(&P[i], &P[i - 1]) : zero3();
            pdf *= pdf_dir(J, &P[i], P[i].type, wi, dirto(&P[i], &P[i + 1]), 0) * geometry_term(&P[i], &P[i + 1]);
        }
    }
    if (t > 0) {
        pdf *= pdf_pos(J, &P[n - 1]) * emitter_pdf(J, &P[n - 1]);
        for (int i = n - 1; i >= s + 1; i--) {
            const v3 wi = i + 1 < n ? dirto(&P[i], &P[i + 1]) : zero3();
            pdf *= pdf_dir(J, &P[i], P[i].type, wi, dirto(&P[i], &P[i - 1]), 0) * geometry_term(&P[i], &P[i - 1]);
        }
    }
    if (merge) pdf *= PI_F * r * r;
    return pdf;
}

/* EvaluateMISWeight_VCM (mode 0), _BDPT (1, connections only), _BDPM (2,
 * merges only): power heuristic, merges counted num_photon_trace_samples
 * times (renderer_vcm.cpp:278-338) */
static float vcm_weight(const bd_job* J, const pvx* P, int n, int s_, int merge_, float r, float n_photon, int mode)
{
    const float ps = vcm_path_pdf(J, P, n, s_, merge_, r);
    float invw = 0.0f;
    for (int s = 0; s <= n; s++)
        for (int type = 0; type < 2; type++) {
            if ((mode == 1 && type == 1) || (mode == 2 && type == 0)) continue;
            const float pi = vcm_path_pdf(J, P, n, s, type, type ? r : 0.0f);
            if (pi > 0.0f) {
                const float q = pi / ps;
                invw += q * q * (type ? n_photon : 1.0f);
            }
        }
    return 1.0f / invw;
}

static int64_t vcm_cell_key(int64_t x, int64_t y, int64_t z)
{
    return ((x + (1 << 20)) << 42) | ((y + (1 << 20)) << 21) | (z + (1 << 20));
}

static int64_t vcm_cell_of(float c) { return (int64_t)floorf(c); }

typedef struct { int64_t key; int32_t ent; } vcm_kv;

static int vcm_kv_cmp(const void* a, const void* b)
{
    const vcm_kv *x = (const vcm_kv*)a, *y = (const vcm_kv*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->ent < y->ent ? -1 : (x->ent > y->ent);
}

static void* vcm_pool_worker(void* arg)
{
    void** a = (void**)arg;
    const bd_job* J = (const bd_job*)a[0];
    const int w = (int)(intptr_t)a[1];
    vcm_ctx* X = (vcm_ctx*)a[2];
    const uint64_t b = X->n_photon * (uint64_t)w / (uint64_t)J->threads;
    const uint64_t e = X->n_photon * (uint64_t)(w + 1) / (uint64_t)J->threads;
    for (uint64_t i = b; i < e; i++) {
        uint64_t rng = vcm_stream(J->seed, X->pass, i, 1);
        X->pool_n[i] = vcm_subpath(J, &rng, DIR_LE, X->pool_v + i * (size_t)J->max_v);
    }
    return NULL;
}

static void vcm_splat(const bd_job* J, const vcm_ctx* X, splat_list* sl, const pvx* P, int n, spd C)
{
    float rx = 0.0f, ry = 0.0f;
    raster_pos(J, dirto(&P[n - 1], &P[n - 2]), &rx, &ry);
    splat_add(sl, pixel_of(J, rx, ry), sscale(sscale(C, (float)(J->W * J->H)), 1.0f / (float)X->n_eye));
}

static void* vcm_eye_worker(void* arg)
{
    void** a = (void**)arg;
    bd_job* J = (bd_job*)a[0];
    const int w = (int)(intptr_t)a[1];
    const vcm_ctx* X = (const vcm_ctx*)a[2];
    const int W = J->W, H = J->H, maxv = J->max_v;
    double* sum = (double*)calloc((size_t)W * H * 3, sizeof(double));
    double* sumsq = (double*)calloc((size_t)W * H * 3, sizeof(double));
    splat_list* sl = (splat_list*)malloc(sizeof(splat_list));
    pvx E[MAXV], L[MAXV], P[2 * MAXV];
    const float r2 = X->r * X->r, nph = (float)X->n_photon;
    const uint64_t b = X->n_eye * (uint64_t)w / (uint64_t)J->threads;
    const uint64_t e = X->n_eye * (uint64_t)(w + 1) / (uint64_t)J->threads;
    for (uint64_t smp = b; smp < e; smp++) {
        sl->n = 0;
        uint64_t rng = vcm_stream(J->seed, X->pass, smp, 2);
        const int nE = vcm_subpath(J, &rng, DIR_EL, E);
        const int nL = vcm_subpath(J, &rng, DIR_LE, L);
        for (int t = 1; t <= nE; t++) {
            if (X->mode != 2) {
                int minS = 2 - t > 0 ? 2 - t : 0;
                if (X->min_v - t > minS) minS = X->min_v - t;
                const int maxS = nL < maxv - t ? nL : maxv - t;
                for (int s = minS; s <= maxS; s++) {
                    /* VCMPath::ConnectSubpaths */
                    int n = 0;
                    if (s == 0) {
                        const pvx* v = &E[t - 1];
                        if (v->prim < 0 || !J->prims[v->prim].is_light) continue;
                        for (int i = t - 1; i >= 0; i--) P[n++] = E[i];
                        P[0].type = T_L;
                    } else {
                        if (!visible(J, L[s - 1].p, E[t - 1].p)) continue;
                        for (int i = 0; i < s; i++) P[n++] = L[i];
                        for (int i = t - 1; i >= 0; i--) P[n++] = E[i];
                    }
                    const spd f = vcm_eval_f(J, P, n, s, 0);
                    if (sblack(f)) continue;
                    const float p = vcm_path_pdf(J, P, n, s, 0, 0.0f);
                    if (p == 0.0f) goto sample_done;
                    const float wgt = vcm_weight(J, P, n, s, 0, X->r, nph, X->mode == 0 ? 0 : 1);
                    vcm_splat(J, X, sl, P, n, sscale(sscale(f, wgt), 1.0f / p));
                }
            }
            if (X->mode != 1) {
                const pvx* vE = &E[t - 1];
                if (is_delta_pos(vE->type)) continue;
                const float ic = X->inv_cell;
                int64_t lo[3], hi[3];
                const float c[3] = {vE->p.x, vE->p.y, vE->p.z};
                for (int k = 0; k < 3; k++) {
                    lo[k] = vcm_cell_of(c[k] * ic - 0.5f - 1e-3f);
                    hi[k] = vcm_cell_of(c[k] * ic + 0.5f + 1e-3f);
                }
                for (int64_t cx = lo[0]; cx <= hi[0]; cx++)
                    for (int64_t cy = lo[1]; cy <= hi[1]; cy++)
                        for (int64_t cz = lo[2]; cz <= hi[2]; cz++) {
                            const int64_t key = vcm_cell_key(cx, cy, cz);
                            size_t l = 0, h = X->nent;
                            while (l < h) {
                                const size_t m = (l + h) / 2;
                                if (X->keys[m] < key) l = m + 1;
                                else h = m;
                            }
                            for (size_t q = l; q < X->nent && X->keys[q] == key; q++) {
                                const int si = X->ent[q] / 64, vi = X->ent[q] % 64;
                                const pvx* pool = X->pool_v + (size_t)si * maxv;
                                const v3 d = sub(pool[vi].p, vE->p);
                                if (!(dot(d, d) < r2)) continue;
                                /* the RangeQuery callback (:729-763) */
                                const int s = vi + 1, n = s + t - 1;
                                if (n < X->min_v || maxv < n) continue;
                                if (is_delta_pos(pool[vi - 1].type) || is_delta_pos(vE->type)) continue;
                                int np = 0;
                                for (int i = 0; i < vi; i++) P[np++] = pool[i];
                                for (int i = t - 1; i >= 0; i--) P[np++] = E[i];
                                const spd f = vcm_eval_f(J, P, np, vi, 1);
                                if (sblack(f)) continue;
                                const float p = vcm_path_pdf(J, P, np, vi, 1, X->r);
                                if (p == 0.0f) continue;
                                const float wgt = vcm_weight(J, P, np, vi, 1, X->r, nph, X->mode == 0 ? 0 : 2);
                                vcm_splat(J, X, sl, P, np, sscale(sscale(f, wgt), 1.0f / p));
                            }
                        }
            }
        }
    sample_done:
        for (int k = 0; k < sl->n; k++)
            for (int ch = 0; ch < 3; ch++) {
                sum[3 * (size_t)sl->pix[k] + ch] += sl->val[k][ch];
                sumsq[3 * (size_t)sl->pix[k] + ch] += sl->val[k][ch] * sl->val[k][ch];
            }
    }
    pthread_mutex_lock(&J->lock);
    for (size_t i = 0; i < (size_t)W * H * 3; i++) { J->sum[i] += sum[i]; J->sumsq[i] += sumsq[i]; }
    pthread_mutex_unlock(&J->lock);
    free(sl);
    free(sum);
    free(sumsq);
    return NULL;
}

uint64_t lmo_render_vcm(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims, int nprims,
                        const lmo_pt_camera* cam, const lmo_vcm_params* prm, uint64_t seed, int threads, double* sum,
                        double* sumsq)
{
    bd_job J;
    bd_job_init(&J, tris, tri_prim, ntri, prims, nprims, cam);
    J.max_v = prm->max_num_vertices;
    J.seed = seed;
    J.threads = threads < 1 ? 1 : threads;
    J.sum = sum;
    J.sumsq = sumsq;
    memset(sum, 0, sizeof(double) * (size_t)J.W * J.H * 3);
    memset(sumsq, 0, sizeof(double) * (size_t)J.W * J.H * 3);
    pthread_mutex_init(&J.lock, NULL);
    uint64_t done = 0;
    if (J.nlights > 0 && J.max_v >= 1 && J.max_v <= MAXV) {
        vcm_ctx X;
        memset(&X, 0, sizeof(X));
        X.mode = prm->mode;
        X.min_v = prm->min_num_vertices;
        X.n_photon = X.mode == 1 ? 0 : prm->num_photon_trace_samples;
        X.n_eye = prm->num_eye_trace_samples;
        X.pool_v = (pvx*)malloc(sizeof(pvx) * (size_t)J.max_v * (X.n_photon ? X.n_photon : 1));
        X.pool_n = (int*)calloc(X.n_photon ? X.n_photon : 1, sizeof(int));
        vcm_kv* kv = (vcm_kv*)malloc(sizeof(vcm_kv) * (size_t)J.max_v * (X.n_photon ? X.n_photon : 1));
        X.keys = (int64_t*)malloc(sizeof(int64_t) * (size_t)J.max_v * (X.n_photon ? X.n_photon : 1));
        X.ent = (int32_t*)malloc(sizeof(int32_t) * (size_t)J.max_v * (X.n_photon ? X.n_photon : 1));
        float r = 0.0f;
        for (uint64_t pass = 0; pass < prm->num_iteration_pass; pass++) {
            r = pass == 0 ? prm->initial_radius : sqrtf((prm->alpha + (float)pass) / (1.0f + (float)pass)) * r;
            X.r = r;
            X.inv_cell = 1.0f / (2.0f * r);
            X.pass = pass;
            X.nent = 0;
            if (X.n_photon) {
                bd_run_workers(&J, vcm_pool_worker, &X);
                for (uint64_t i = 0; i < X.n_photon; i++)
                    for (int k = 1; k < X.pool_n[i]; k++) {
                        const pvx* v = &X.pool_v[i * (size_t)J.max_v + k];
                        if (is_delta_pos(v->type) || is_delta_dir(&J, v, v->type)) continue;
                        kv[X.nent].key = vcm_cell_key(vcm_cell_of(v->p.x * X.inv_cell), vcm_cell_of(v->p.y * X.inv_cell),
                                                      vcm_cell_of(v->p.z * X.inv_cell));
                        kv[X.nent].ent = (int32_t)(i * 64 + (uint64_t)k);
                        X.nent++;
                    }
                qsort(kv, X.nent, sizeof(vcm_kv), vcm_kv_cmp);
                for (size_t q = 0; q < X.nent; q++) { X.keys[q] = kv[q].key; X.ent[q] = kv[q].ent; }
            }
            bd_run_workers(&J, vcm_eye_worker, &X);
            done += X.n_eye;
        }
        free(X.pool_v); free(X.pool_n); free(kv); free(X.keys); free(X.ent);
    }
    pthread_mutex_destroy(&J.lock);
    bd_job_release(&J);
    return done;
}
