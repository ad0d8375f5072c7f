// Bidirectional path tracing on the GPU: the form of renderer::bdpt.
//
// Reference estimator (src/liblightmetrica/renderer/renderer_bdpt.cpp):
//   * a light subpath and an eye subpath per sample (Subpath::Sample, :80-220):
//     after the first vertex every step stores a BSDF-sampled vertex and a
//     "direct" vertex (the opposite endpoint's emitter sampled from the
//     previous vertex, kept only when visible); roulette 0.5 after each step;
//   * every strategy (s, t, direct) with direct only for s = 0 or t = 0
//     (Render, :841-998) is connected (Path::Connect, :233-333), weighted by
//     the power heuristic over all strategies of the same full path
//     (:747-784, EvaluatePDF :628-703), divided by the roulette selection
//     probability 0.5^(max(0,s-2)+max(0,t-2)) (:348-368) and splatted at
//     the raster position of the path's last segment;
//   * light::area draws its emission direction from the same 2D sample as the
//     position (light_area.cpp:73-80) and the pinhole is a delta position, so
//     t = 0 strategies carry no weight -- both kept as the reference has them.
//
// GPU structure: one thread per sample, the two subpaths in per-thread local
// arrays (at most kMaxV vertices each), rays traced with the per-thread
// traversal of traverse.cuh.  Contributions that land in the sample's own
// pixel are summed in registers and splatted once; others (light-to-camera
// connections) are splatted where they land.  Eye subpaths start from
// per-pixel stratified raster positions; random numbers are Philox keyed by
// (seed, sample).
#include "bsdf.cuh"
#include "rng.cuh"
#include "scene.cuh"
#include "traverse.cuh"

namespace lmgpu {
namespace {

constexpr int kMaxV = 16;
constexpr int kBdptThreads = 128;
constexpr uint32_t kKeyBdpt = 0x42445054u;

// SurfaceInteractionType (surfaceinteraction.h:39-52)
enum : int { T_D = 1, T_G = 2, T_S = 4, T_L = 8, T_E = 16 };
enum : int { DIR_LE = 0, DIR_EL = 1 };

struct PV {  // 32 bytes
    float3 p, n;
    int prim;  // -1: the sensor
    short type;
    short degen;
};

struct SV {
    PV sv, direct;
    int has_sv, has_direct;
};

struct Rng {
    uint32_t c0, c1, seed, ctr;
    float buf[4];
    int left;
};

__device__ __forceinline__ float rnd(Rng& r)
{
    if (r.left == 0) {
        const Philox4x32 x = philox4x32_10(r.c0, r.c1, r.ctr++, 0u, r.seed, kKeyBdpt);
        for (int k = 0; k < 4; k++) r.buf[k] = u01(x.v[k]);
        r.left = 4;
    }
    return r.buf[--r.left];
}

struct Ctx {
    SceneGPU sc;
    LightsGPU lights;
    CameraGPU cam;
    TraceView tv;
    int max_v;     // subpath vertices, at most kMaxV
    int max_path;  // full-path vertices (the reference's max_num_vertices; -1 = unbounded)
};

__device__ __forceinline__ float3 zero3() { return f3(0.0f, 0.0f, 0.0f); }
__device__ __forceinline__ float3 dirto(const PV& a, const PV& b) { return normalize3(b.p - a.p); }

__device__ __forceinline__ int bsdf_type(int bsdf)
{
    return bsdf == LMGPU_BSDF_DIFFUSE ? T_D : bsdf == LMGPU_BSDF_DIELECTRIC ? T_S : bsdf == LMGPU_BSDF_COOK_TORRANCE ? T_G : 0;
}

__device__ __forceinline__ float3 to_local(float3 n, float3 w)
{
    float3 b, c;
    basis(n, b, c);
    return f3(dot3(w, b), dot3(w, c), dot3(w, n));
}

// Sensor_Pinhole::RasterPosition / Importance (sensor_pinhole.cpp:137-185)
__device__ __forceinline__ bool raster_pos(const CameraGPU& cam, float3 wo, float& rx, float& ry)
{
    const float ex = dot3(cam.vx, wo), ey = dot3(cam.vy, wo), ez = dot3(cam.vz, wo);
    if (ez >= 0.0f) return false;
    rx = (-ex / ez / cam.tan_fov / cam.aspect + 1.0f) * 0.5f;
    ry = (-ey / ez / cam.tan_fov + 1.0f) * 0.5f;
    return !(rx < 0.0f || rx > 1.0f || ry < 0.0f || ry > 1.0f);
}

__device__ __forceinline__ float importance(const CameraGPU& cam, float3 wo)
{
    float rx, ry;
    if (!raster_pos(cam, wo, rx, ry)) return 0.0f;
    const float ic = 1.0f / -dot3(cam.vz, wo);
    return ic * ic * ic / (cam.tan_fov * cam.tan_fov * cam.aspect * 4.0f);
}

struct Spd {
    float c[3];
};
__device__ __forceinline__ Spd S1(float v) { return Spd{{v, v, v}}; }
__device__ __forceinline__ bool black(const Spd& a) { return a.c[0] == 0.0f && a.c[1] == 0.0f && a.c[2] == 0.0f; }

// Primitive::EvaluateDirection (primitive.h:147-170) for the vertex roles used here.
__device__ __noinline__ Spd eval_dir(const Ctx& C, const PV& v, int type, float3 wi, float3 wo, int dir, bool evalDelta)
{
    if (type & T_E) return S1(importance(C.cam, wo));
    if (type & T_L) {
        if (dot3(wo, v.n) <= 0.0f) return S1(0.0f);
        const PrimGPU& P = C.sc.prims[v.prim];
        return Spd{{P.Le[0], P.Le[1], P.Le[2]}};
    }
    if (v.prim < 0) return S1(0.0f);
    const PrimGPU P = C.sc.prims[v.prim];
    const float3 lwi = to_local(v.n, wi), lwo = to_local(v.n, wo);
    // BSDFUtils::ShadingNormalCorrection (bsdfutils.h:55-66) with sn = gn
    const float wig = dot3(wi, v.n), wog = dot3(wo, v.n);
    const float snc = (wig * wig <= 0.0f || wog * wog <= 0.0f) ? 0.0f : 1.0f;
    Spd r = S1(0.0f);
    if (P.bsdf == LMGPU_BSDF_DIFFUSE) {
        if (lwi.z <= 0.0f || lwo.z <= 0.0f) return r;
        for (int k = 0; k < 3; k++) r.c[k] = P.R[k] * 0.31830988618379067f * snc;
    } else if (P.bsdf == LMGPU_BSDF_DIELECTRIC) {
        if (evalDelta) return r;
        float etaI = P.eta1, etaT = P.eta2;
        if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
        const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
        if (lwi.z * lwo.z >= 0.0f) {
            for (int k = 0; k < 3; k++) r.c[k] = P.R[k] * Fr * snc;
        } else {
            const float eta = etaI / etaT;
            const float rc = dir == DIR_EL ? eta : 1.0f;
            for (int k = 0; k < 3; k++) r.c[k] = P.R[k] * (1.0f - Fr) * snc * rc * rc;
        }
    } else if (P.bsdf == LMGPU_BSDF_COOK_TORRANCE) {
        if (lwi.z <= 0.0f || lwo.z <= 0.0f) return r;
        const float3 H = normalize3(lwi + lwo);
        const float D = ggx_d(H, P.roughness);
        const float woH = fabsf(dot3(lwo, H));
        const float G = fminf(1.0f, fminf(2.0f * H.z * lwo.z / woH, 2.0f * H.z * lwi.z / woH));
        const float cih = dot3(lwi, H);
        for (int k = 0; k < 3; k++)
            r.c[k] = P.R[k] * D * G * fresnel_conductor(cih, P.ct_eta[k], P.ct_k[k]) / (4.0f * lwi.z) / lwo.z * snc;
    }
    return r;
}

// EvaluateDirectionPDF, projected solid angle measure.
__device__ __noinline__ float pdf_dir(const Ctx& C, const PV& v, int type, float3 wi, float3 wo)
{
    if (type & T_E) return importance(C.cam, wo);
    if (type & T_L) return dot3(wo, v.n) <= 0.0f ? 0.0f : 0.31830988618379067f;
    if (v.prim < 0) return 0.0f;
    const PrimGPU P = C.sc.prims[v.prim];
    const float3 lwi = to_local(v.n, wi), lwo = to_local(v.n, wo);
    if (P.bsdf == LMGPU_BSDF_DIFFUSE) return (lwi.z <= 0.0f || lwo.z <= 0.0f) ? 0.0f : 0.31830988618379067f;
    if (P.bsdf == LMGPU_BSDF_DIELECTRIC) {
        float etaI = P.eta1, etaT = P.eta2;
        if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
        const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
        return lwi.z * lwo.z >= 0.0f ? Fr : 1.0f - Fr;
    }
    if (P.bsdf == LMGPU_BSDF_COOK_TORRANCE) {
        if (lwi.z <= 0.0f || lwo.z <= 0.0f) return 0.0f;
        const float3 H = normalize3(lwi + lwo);
        return ggx_d(H, P.roughness) * H.z / (4.0f * dot3(lwo, H)) / lwo.z;
    }
    return 0.0f;
}

__device__ __forceinline__ bool delta_dir(const Ctx& C, const PV& v, int type)
{
    if (type & (T_E | T_L)) return false;
    return v.prim >= 0 && C.sc.prims[v.prim].bsdf == LMGPU_BSDF_DIELECTRIC;
}

// EvaluatePositionGiven{Direction,PreviousPosition}PDF (area measure) and
// Scene3::EvaluateEmitterPDF (scene3.cpp:525-539).
__device__ __forceinline__ float pdf_pos(const Ctx& C, const PV& v)
{
    if ((v.type & T_E) || v.prim < 0) return 1.0f;
    const int l = C.lights.prim_light[v.prim];
    return l < 0 ? 0.0f : C.lights.inv_area[l];
}
__device__ __forceinline__ float emitter_pdf(const Ctx& C, const PV& v)
{
    return v.prim < 0 ? 1.0f : 1.0f / (float)C.lights.count;
}

// RenderUtils::GeometryTerm (renderutils.h:46-56)
__device__ __forceinline__ float geometry_term(const PV& a, const PV& b)
{
    float3 d = b.p - a.p;
    const float l2 = dot3(d, d);
    d = d * (1.0f / sqrtf(l2));
    float t = 1.0f;
    if (!a.degen) t *= fabsf(dot3(a.n, d));
    if (!b.degen) t *= fabsf(dot3(b.n, d));
    return t / l2;
}

// Light selection, area-weighted triangle (Distribution1D::SampleReuse,
// dist.h:71-77), uniform point (TriangleUtils::SampleTriangleMesh).
__device__ __noinline__ void sample_light(const Ctx& C, float us, float ux, float uy, PV& v)
{
    const int nl = C.lights.count;
    int li = (int)(us * (float)nl);
    li = li < 0 ? 0 : (li > nl - 1 ? nl - 1 : li);
    const int off = C.lights.tri_off[li];
    const int nt = C.lights.tri_off[li + 1] - off;
    const float* cdf = C.lights.cdf + off + li;
    int lo = 0, hi = nt + 1;
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (cdf[m] <= ux) lo = m + 1;
        else hi = m;
    }
    int i = lo - 1;
    i = i < 0 ? 0 : (i > nt - 1 ? nt - 1 : i);
    const float u2x = (ux - cdf[i]) / (cdf[i + 1] - cdf[i]);
    const float s = sqrtf(fmaxf(u2x, 0.0f));
    const float bx = 1.0f - s, by = uy * s;
    const float* T = C.sc.tris + 9 * (size_t)C.lights.tris[off + i];
    const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
    v.p = p1 * (1.0f - bx - by) + p2 * bx + p3 * by;
    v.n = normalize3(cross3(p2 - p1, p3 - p1));
    v.prim = C.lights.prims[li];
    v.type = T_L;
    v.degen = 0;
}

__device__ __forceinline__ void sensor_vertex(const Ctx& C, PV& v)
{
    v.p = C.cam.eye;
    v.n = C.cam.vz;
    v.prim = -1;
    v.type = T_E;
    v.degen = 1;
}

// One out-of-line copy of the traversal for every ray the kernel traces.
__device__ __noinline__ bool trace_one(const TraceView& tv, float3 o, float tmin, float3 d, float tmax, bool anyhit,
                                       float& t, int& id, float& b1, float& b2)
{
    return trace_single(tv, o, tmin, d, tmax, anyhit, t, id, b1, b2);
}

__device__ __noinline__ bool trace_vertex(const Ctx& C, float3 o, float3 d, PV& v)
{
    float t, b1, b2;
    int id;
    if (!trace_one(C.tv, o, 1e-4f, d, FLT_MAX, false, t, id, b1, b2)) return false;
    const float* T = C.sc.tris + 9 * (size_t)id;
    const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
    v.p = o + d * t;
    v.n = normalize3(cross3(p2 - p1, p3 - p1));
    v.prim = C.sc.tri_prim[id];
    v.type = bsdf_type(C.sc.prims[v.prim].bsdf);
    v.degen = 0;
    return true;
}

// Scene3::Visible (scene3.h:107-116): [EpsIsect, L (1 - EpsIsect)]
__device__ __noinline__ bool visible(const Ctx& C, float3 a, float3 b)
{
    float3 d = b - a;
    const float L = sqrtf(dot3(d, d));
    d = d * (1.0f / L);
    float t, b1, b2;
    int id;
    return !trace_one(C.tv, a, 1e-4f, d, L * (1.0f - 1e-4f), true, t, id, b1, b2);
}

// BSDF SampleDirection; false where the reference leaves wo unset.
__device__ __noinline__ bool sample_dir(const Ctx& C, const PV& v, float3 wi, float u0, float u1, float uc, float3& wo)
{
    if (v.prim < 0) return false;
    const PrimGPU P = C.sc.prims[v.prim];
    float3 b, c;
    basis(v.n, b, c);
    const float3 lwi = f3(dot3(wi, b), dot3(wi, c), dot3(wi, v.n));
    float3 lwo;
    if (P.bsdf == LMGPU_BSDF_DIFFUSE) {
        if (lwi.z <= 0.0f) return false;
        lwo = cosine_hemisphere(u0, u1);
    } else if (P.bsdf == LMGPU_BSDF_DIELECTRIC) {
        float etaI = P.eta1, etaT = P.eta2;
        if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
        const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
        if (uc <= Fr) {
            lwo = f3(-lwi.x, -lwi.y, lwi.z);
        } else {
            const float eta = etaI / etaT;
            const float ct2 = 1.0f - eta * eta * (1.0f - lwi.z * lwi.z);
            lwo = f3(-eta * lwi.x, -eta * lwi.y, sqrtf(fmaxf(ct2, 0.0f)) * (lwi.z > 0.0f ? -1.0f : 1.0f));
        }
    } else if (P.bsdf == LMGPU_BSDF_COOK_TORRANCE) {
        if (lwi.z <= 0.0f) return false;
        const float3 H = ggx_sample(u0, u1, P.roughness);
        lwo = (lwi * -1.0f) - H * (2.0f * -dot3(lwi, H));
        if (lwo.z <= 0.0f) return false;
    } else {
        return false;
    }
    wo = b * lwo.x + c * lwo.y + v.n * lwo.z;
    return true;
}

// Subpath::Sample (renderer_bdpt.cpp:80-220).  For the eye subpath the first
// direction comes from the stratified raster position (rx0, ry0).
__device__ __noinline__ int sample_subpath(const Ctx& C, Rng& rng, int dir, float rx0, float ry0, SV* out)
{
    int n = 0;
    float3 initWo = zero3();
    for (int step = 0; step < C.max_v; step++) {
        if (step == 0) {
            PV v;
            if (dir == DIR_LE) {
                const float us = rnd(rng), a0 = rnd(rng), a1 = rnd(rng);
                sample_light(C, us, a0, a1, v);
                // direction from the same 2D sample as the position (light_area.cpp:73-80)
                const float3 l = cosine_hemisphere(a0, a1);
                float3 b, c;
                basis(v.n, b, c);
                initWo = b * l.x + c * l.y + v.n * l.z;
            } else {
                sensor_vertex(C, v);
                initWo = camera_dir(C.cam, rx0, ry0);
            }
            out[n].sv = v;
            out[n].has_sv = 1;
            out[n].has_direct = 0;
            n++;
            continue;
        }
        const PV pv = out[n - 1].sv;
        SV nv;
        nv.has_sv = 0;
        nv.has_direct = 0;
        {
            const float3 wi = n > 1 ? dirto(pv, out[n - 2].sv) : zero3();
            const float u0 = rnd(rng), u1 = rnd(rng), uc = rnd(rng);
            float3 wo = zero3();
            bool ok = true;
            if (step == 1) wo = initWo;
            else ok = sample_dir(C, pv, wi, u0, u1, uc, wo);
            if (ok && !black(eval_dir(C, pv, pv.type, wi, wo, dir, false)) && trace_vertex(C, pv.p, wo, nv.sv))
                nv.has_sv = 1;
        }
        {
            const float us = rnd(rng), a0 = rnd(rng), a1 = rnd(rng);
            PV v;
            if (dir == DIR_LE) sensor_vertex(C, v);
            else sample_light(C, us, a0, a1, v);
            if (visible(C, pv.p, v.p)) {
                nv.direct = v;
                nv.has_direct = 1;
            }
        }
        if (nv.has_sv || nv.has_direct) out[n++] = nv;
        if (!nv.has_sv) break;
        if (rnd(rng) > 0.5f) break;
    }
    return n;
}

// Path::Connect (renderer_bdpt.cpp:233-333)
__device__ __noinline__ int connect(const Ctx& C, int s, int t, bool direct, const SV* L, const SV* E, PV* P)
{
    int n = 0;
    if (s == 0 && t > 0) {
        if (!direct) {
            if (!E[t - 1].has_sv) return 0;
            const int pr = E[t - 1].sv.prim;
            if (pr < 0 || !C.sc.prims[pr].is_light) return 0;
            for (int i = t - 1; i >= 0; i--) P[n++] = E[i].sv;
        } else {
            if (!E[t - 1].has_direct) return 0;
            P[n++] = E[t - 1].direct;
            for (int i = t - 2; i >= 0; i--) P[n++] = E[i].sv;
        }
        P[0].type = T_L;
    } else if (s > 0 && t == 0) {
        if (!direct) return 0;  // a light subpath vertex is never the pinhole
        if (!L[s - 1].has_direct) return 0;
        for (int i = 0; i < s - 1; i++) P[n++] = L[i].sv;
        P[n++] = L[s - 1].direct;
        P[n - 1].type = T_E;
    } else {
        if (!L[s - 1].has_sv || !E[t - 1].has_sv) return 0;
        if (!visible(C, L[s - 1].sv.p, E[t - 1].sv.p)) return 0;
        for (int i = 0; i < s; i++) P[n++] = L[i].sv;
        for (int i = t - 1; i >= 0; i--) P[n++] = E[i].sv;
    }
    return n;
}

// EvaluateUnweightContribution (:489-591) with EvaluateCst (:375-406).
__device__ __noinline__ Spd unweighted(const Ctx& C, const PV* P, int n, int s, bool direct)
{
    const int t = n - s;
    Spd a = S1(1.0f);
    if (s > 0) {
        a = S1(1.0f / pdf_pos(C, P[0]) / emitter_pdf(C, P[0]));
        for (int i = 0; i < s - 1; i++) {
            const float3 wi = i >= 1 ? dirto(P[i], P[i - 1]) : zero3(), wo = dirto(P[i], P[i + 1]);
            const bool dl = t == 0 && i == s - 2 && direct;
            const Spd fs = eval_dir(C, P[i], P[i].type, wi, wo, DIR_LE, dl);
            if (black(fs)) return S1(0.0f);
            const float pdf = dl ? pdf_pos(C, P[i + 1]) / geometry_term(P[i + 1], P[i]) * emitter_pdf(C, P[i + 1])
                                 : pdf_dir(C, P[i], P[i].type, wi, wo);
            for (int k = 0; k < 3; k++) a.c[k] *= fs.c[k] / pdf;
        }
    }
    if (black(a)) return a;
    if (t > 0) {
        const float ae = 1.0f / pdf_pos(C, P[n - 1]) / emitter_pdf(C, P[n - 1]);
        for (int k = 0; k < 3; k++) a.c[k] *= ae;
        for (int i = n - 1; i > s; i--) {
            const float3 wi = i < n - 1 ? dirto(P[i], P[i + 1]) : zero3(), wo = dirto(P[i], P[i - 1]);
            const bool dl = s == 0 && i == 1 && direct;
            const Spd fs = eval_dir(C, P[i], P[i].type, wi, wo, DIR_EL, dl);
            if (black(fs)) return S1(0.0f);
            const float pdf = dl ? pdf_pos(C, P[i - 1]) / geometry_term(P[i - 1], P[i]) * emitter_pdf(C, P[i - 1])
                                 : pdf_dir(C, P[i], P[i].type, wi, wo);
            for (int k = 0; k < 3; k++) a.c[k] *= fs.c[k] / pdf;
        }
    }
    if (black(a)) return a;
    // Cst
    Spd cst;
    if (s == 0 && t > 0) {
        cst = eval_dir(C, P[0], P[0].type, zero3(), dirto(P[0], P[1]), DIR_EL, false);
    } else if (s > 0 && t == 0) {
        cst = S1(0.0f);  // EvaluatePosition(evalDelta = true) of the pinhole is 0
    } else {
        const PV& vL = P[s - 1];
        const PV& vE = P[s];
        const Spd fL = eval_dir(C, vL, vL.type, s - 2 >= 0 ? dirto(vL, P[s - 2]) : zero3(), dirto(vL, vE), DIR_LE, true);
        const Spd fE = eval_dir(C, vE, vE.type, s + 1 < n ? dirto(vE, P[s + 1]) : zero3(), dirto(vE, vL), DIR_EL, true);
        const float G = geometry_term(vL, vE);
        for (int k = 0; k < 3; k++) cst.c[k] = fL.c[k] * G * fE.c[k];
    }
    for (int k = 0; k < 3; k++) a.c[k] *= cst.c[k];
    return a;
}

// Samplable + EvaluatePDF (:593-703) for every strategy of one full path,
// and the power-heuristic weight of strategy (s_, d_) over them
// (MISWeight_PowerHeuristics, :747-784).  EvaluatePDF(s, d) is the product
// of the endpoint terms and of one factor per vertex,
//   light side  fL[i] = pdf_dir(P[i] -> P[i+1]) G(P[i], P[i+1]),  i < s - 1
//   eye side    fE[i] = pdf_dir(P[i] -> P[i-1]) G(P[i], P[i-1]),  i > s
// with the direct strategies swapping the factor next to the sampled
// endpoint for that endpoint's positional pdf.  The factors are evaluated
// once per path and combined through prefix / suffix products, so every
// strategy's pdf costs O(1) instead of O(n).
__device__ __noinline__ float mis_weight(const Ctx& C, const PV* P, int n, int s_, bool d_)
{
    float preL[2 * kMaxV + 1], sufE[2 * kMaxV + 1];
    const float posL = pdf_pos(C, P[0]) * emitter_pdf(C, P[0]);
    const float posE = pdf_pos(C, P[n - 1]) * emitter_pdf(C, P[n - 1]);
    // preL[k] = posL * prod_{i < k} fL[i], k = 0 .. n - 1
    preL[0] = posL;
    for (int i = 0; i + 1 < n; i++) {
        const float f = pdf_dir(C, P[i], P[i].type, i >= 1 ? dirto(P[i], P[i - 1]) : zero3(), dirto(P[i], P[i + 1])) *
                        geometry_term(P[i], P[i + 1]);
        preL[i + 1] = preL[i] * f;
    }
    // sufE[k] = posE * prod_{i >= k} fE[i], k = n .. 1
    sufE[n] = posE;
    for (int i = n - 1; i >= 1; i--) {
        const float f = pdf_dir(C, P[i], P[i].type, i + 1 < n ? dirto(P[i], P[i + 1]) : zero3(),
                                dirto(P[i], P[i - 1])) *
                        geometry_term(P[i], P[i - 1]);
        sufE[i] = sufE[i + 1] * f;
    }
    auto pdf = [&](int s, bool d) -> float {
        const int t = n - s;
        if (s > 0 && t > 0 && d) return 0.0f;
        if (t == 0 && s > 0 && d && delta_dir(C, P[n - 2], P[n - 2].type)) return 0.0f;
        if (s == 0 && t > 0 && d && delta_dir(C, P[1], P[1].type)) return 0.0f;
        if (s == 0 && t > 0) {
            if (P[0].type & T_E) return 0.0f;
        } else if (s > 0 && t == 0) {
            if (P[n - 1].type & T_E) return 0.0f;
        } else if (delta_dir(C, P[s - 1], P[s - 1].type) || delta_dir(C, P[s], P[s].type)) {
            return 0.0f;
        }
        float pl = 1.0f, pe = 1.0f;
        if (s > 0) pl = (t == 0 && d) ? preL[s - 2] * posE : preL[s - 1];
        if (t > 0) pe = (s == 0 && d) ? sufE[2] * posL : sufE[s + 1];
        return pl * pe;
    };
    const float ps = pdf(s_, d_);
    float inv = 0.0f;
    for (int s = 0; s <= n; s++)
        for (int d = 0; d < 2; d++) {
            if (s > 0 && n - s > 0 && d) continue;
            const float pi = pdf(s, d != 0);
            if (pi > 0.0f) {
                const float r = pi / ps;
                inv += r * r;
            }
        }
    return 1.0f / inv;
}

__device__ __forceinline__ void splat_px(double* film, double* film_sq, uint32_t pix, const float c[3])
{
    for (int k = 0; k < 3; k++) {
        if (c[k] != 0.0f) {
            atomicAdd(&film[3 * (size_t)pix + k], (double)c[k]);
            atomicAdd(&film_sq[3 * (size_t)pix + k], (double)c[k] * (double)c[k]);
        }
    }
}

__global__ void __launch_bounds__(kBdptThreads) k_bdpt(Ctx C, uint64_t p0, uint32_t count, uint32_t seed,
                                                       double* __restrict__ film, double* __restrict__ film_sq,
                                                       double* __restrict__ film_x, double* __restrict__ film_x_sq)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint64_t p = p0 + i;
    const uint32_t W = (uint32_t)C.cam.width, H = (uint32_t)C.cam.height;
    const uint32_t pixel = (uint32_t)(p % ((uint64_t)W * H));
    Rng rng;
    rng.c0 = (uint32_t)p;
    rng.c1 = (uint32_t)(p >> 32);
    rng.seed = seed;
    rng.ctr = 0;
    rng.left = 0;
    const float rx0 = ((float)(pixel % W) + rnd(rng)) / (float)W;
    const float ry0 = ((float)(pixel / W) + rnd(rng)) / (float)H;
    SV L[kMaxV], E[kMaxV];
    PV P[2 * kMaxV];
    const int nL = sample_subpath(C, rng, DIR_LE, 0.0f, 0.0f, L);
    const int nE = sample_subpath(C, rng, DIR_EL, rx0, ry0, E);
    float own[3] = {0.0f, 0.0f, 0.0f};
    for (int n = 2; n <= nE + nL; n++) {
        if (C.max_path >= 0 && n > C.max_path) continue;
        const int minS = n - nE > 0 ? n - nE : 0;
        const int maxS = nL < n ? nL : n;
        for (int s = minS; s <= maxS; s++)
            for (int d = 0; d < 2; d++) {
                const int t = n - s;
                if (s > 0 && t > 0 && d) continue;
                const int np = connect(C, s, t, d != 0, L, E, P);
                if (!np) continue;
                const Spd cs = unweighted(C, P, np, s, d != 0);
                if (black(cs)) continue;
                const float w = mis_weight(C, P, np, s, d != 0);
                float sel = 1.0f;
                for (int q = 1; q < s - 1; q++) sel *= 0.5f;
                for (int q = 1; q < t - 1; q++) sel *= 0.5f;
                float c[3];
                bool any = false;
                for (int k = 0; k < 3; k++) {
                    c[k] = cs.c[k] * w / sel;
                    any = any || (c[k] != 0.0f && c[k] == c[k]);
                }
                if (!any || !(w == w)) continue;
                float rx = 0.0f, ry = 0.0f;
                raster_pos(C.cam, dirto(P[np - 1], P[np - 2]), rx, ry);
                int ix = (int)(rx * (float)W), iy = (int)(ry * (float)H);
                ix = ix < 0 ? 0 : (ix > (int)W - 1 ? (int)W - 1 : ix);
                iy = iy < 0 ? 0 : (iy > (int)H - 1 ? (int)H - 1 : iy);
                const uint32_t pix = (uint32_t)iy * W + (uint32_t)ix;
                if (pix == pixel) {
                    for (int k = 0; k < 3; k++) own[k] += c[k];
                } else {
                    splat_px(film_x, film_x_sq, pix, c);
                }
            }
    }
    splat_px(film, film_sq, pixel, own);
}

}  // namespace

int render_bdpt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream)
{
    const uint32_t W = (uint32_t)sc->cam.width, H = (uint32_t)sc->cam.height;
    const uint64_t npix = (uint64_t)W * H;
    const uint64_t total = npix * prm->spp;
    if (total == 0) return LMGPU_OK;
    if (sc->lights.count == 0) {
        set_error("lmgpu_render_bdpt: the scene has no area light");
        return LMGPU_ERR_INVALID;
    }
    int rc = clear_film(sc, npix, stream);
    if (rc) return rc;
    // The kernel keeps both subpaths in per-thread local memory (~4 KB):
    // raise the per-thread stack limit once, up front, rather than have the
    // launch resize the device's local-memory pool.
    cudaFuncAttributes fa{};
    LMGPU_CUDA_TRY(cudaFuncGetAttributes(&fa, k_bdpt));
    size_t stack = 0;
    LMGPU_CUDA_TRY(cudaDeviceGetLimit(&stack, cudaLimitStackSize));
    if (stack < fa.localSizeBytes) LMGPU_CUDA_TRY(cudaDeviceSetLimit(cudaLimitStackSize, fa.localSizeBytes));
    Ctx C;
    C.sc = scene_view(sc);
    C.lights = sc->lights;
    C.cam = sc->cam;
    C.tv.nodes = sc->accel->nodes;
    C.tv.tris = sc->accel->tris;
    C.tv.num_nodes = sc->ntri > 0 ? (uint32_t)sc->accel->num_wide : 0u;
    C.tv.num_tris = (uint32_t)sc->ntri;
    C.tv.status = sc->accel->status;
    C.max_v = prm->max_num_vertices < 0 || prm->max_num_vertices > kMaxV ? kMaxV : prm->max_num_vertices;
    C.max_path = prm->max_num_vertices;
    const uint64_t wave = 1ull << 20;
    for (uint64_t p0 = 0; p0 < total; p0 += wave) {
        const uint32_t n = (uint32_t)((total - p0) < wave ? (total - p0) : wave);
        k_bdpt<<<(n + kBdptThreads - 1) / kBdptThreads, kBdptThreads, 0, stream>>>(C, p0, n, prm->seed, sc->film,
                                                                                  sc->film_sq, sc->film_x,
                                                                                  sc->film_x_sq);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
    }
    return finalize_film(sc, prm->spp, d_image, d_variance, stream);
}

}  // namespace lmgpu
