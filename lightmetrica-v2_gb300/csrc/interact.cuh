// Surface interactions shared by the GPU renderers (Primitive's dispatch,
// primitive.h:84-199): path vertices, the pinhole sensor's raster position
// and importance, BSDF evaluate / pdf / sample for both transport
// directions, the area lights' position sampling and pdfs, and the
// geometry term.  Kept out of line (__noinline__) where large, so divergent
// lanes of a kernel share one copy of the code.
#pragma once

#include "bsdf.cuh"

namespace lmgpu {
namespace {

// SurfaceInteractionType (surfaceinteraction.h:39-52)
enum : int { T_D = 1, T_G = 2, T_S = 4, T_L = 8, T_E = 16 };
enum : int { DIR_LE = 0, DIR_EL = 1 };

struct PV {  // 32 bytes
    float3 p, n;
    int prim;  // -1: the sensor
    short type;
    short degen;
};

// Read-only view of a scene for the renderers' kernels (passed by value).
struct Ctx {
    SceneGPU sc;
    LightsGPU lights;
    CameraGPU cam;
    int max_v;     // BDPT: subpath vertices (capped); PT: unused
    int max_path;  // full-path vertices (the reference's max_num_vertices; -1 = unbounded)
    int mis = 0;   // BDPT weight: 0 power heuristic, 1 one over the number of samplable strategies
    int min_path = 0;  // full paths with fewer vertices contribute nothing (the reference's min_num_vertices)
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

// Appends a pending light-sample contribution (shadow ray v -> L) with
// warp-aggregated atomics (a block-aggregated form measured 2 % slower on
// ptmis); every lane of the warp must call it.
__device__ __forceinline__ void append_nee(bool has, const PV& v, const PV& L, const float c[3], uint32_t pix,
                                           uint32_t path, float4* __restrict__ rays, float4* __restrict__ rec,
                                           uint32_t* __restrict__ rec_path, uint32_t* __restrict__ count)
{
    const unsigned m = __ballot_sync(0xffffffffu, has);
    if (m == 0u) return;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (has) {
        const uint32_t o = base + __popc(m & ((1u << lane) - 1u));
        float3 d = L.p - v.p;
        const float len = sqrtf(dot3(d, d));
        d = d * (1.0f / len);
        rays[2 * o] = make_float4(v.p.x, v.p.y, v.p.z, 1e-4f);
        rays[2 * o + 1] = make_float4(d.x, d.y, d.z, len * (1.0f - 1e-4f));
        rec[o] = make_float4(c[0], c[1], c[2], __uint_as_float(pix));
        rec_path[o] = path;
    }
}

__device__ __forceinline__ uint32_t pixel_at(const CameraGPU& cam, float rx, float ry)
{
    int ix = (int)(rx * (float)cam.width), iy = (int)(ry * (float)cam.height);
    ix = ix < 0 ? 0 : (ix > cam.width - 1 ? cam.width - 1 : ix);
    iy = iy < 0 ? 0 : (iy > cam.height - 1 ? cam.height - 1 : iy);
    return (uint32_t)iy * (uint32_t)cam.width + (uint32_t)ix;
}

}  // namespace
}  // namespace lmgpu
