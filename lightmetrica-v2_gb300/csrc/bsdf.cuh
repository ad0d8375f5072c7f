// Device-side surface interactions shared by the GPU renderers: vector
// helpers, the shading frame, the pinhole camera direction and the four BSDFs
// of the reference (bsdf::null, bsdf::diffuse, bsdf::flesnel,
// bsdf::cook_torrance), sampled for the eye-to-light transport direction.
#pragma once

#include "scene.cuh"

namespace lmgpu {

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return f3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float3 normalize3(float3 a) { return a * rsqrtf(dot3(a, a)); }

// Sampler::UniformConcentricDiskSample + CosineSampleHemisphere (sampler.h:44-67).
__device__ __forceinline__ float3 cosine_hemisphere(float u0, float u1)
{
    const float vx = 2.0f * u0 - 1.0f, vy = 2.0f * u1 - 1.0f;
    float sx = 0.0f, sy = 0.0f;
    if (!(vx == 0.0f && vy == 0.0f)) {
        const float qp = 0.78539816339744831f;  // pi / 4
        float r, theta;
        if (vx > -vy) {
            if (vx > vy) { r = vx; theta = qp * __fdividef(vy, vx); }
            else { r = vy; theta = qp * (2.0f - __fdividef(vx, vy)); }
        } else {
            if (vx < vy) { r = -vx; theta = qp * (4.0f + __fdividef(vy, vx)); }
            else { r = -vy; theta = qp * (6.0f - __fdividef(vx, vy)); }
        }
        float s, c;
        __sincosf(theta, &s, &c);
        sx = r * c;
        sy = r * s;
    }
    const float z2 = 1.0f - sx * sx - sy * sy;
    return f3(sx, sy, sqrtf(fmaxf(z2, 0.0f)));
}

// Math::OrthonormalBasis (math.h:2355-2359): columns (b, c, a) map local to world.
__device__ __forceinline__ void basis(float3 a, float3& b, float3& c)
{
    c = fabsf(a.x) > fabsf(a.y) ? normalize3(f3(a.z, 0.0f, -a.x)) : normalize3(f3(0.0f, a.z, -a.y));
    b = cross3(c, a);
}

// Pinhole direction for raster position (rx, ry) in [0,1]^2 (sensor_pinhole.cpp:86-89).
__device__ __forceinline__ float3 camera_dir(const CameraGPU& cam, float rx, float ry)
{
    const float px = 2.0f * rx - 1.0f, py = 2.0f * ry - 1.0f;
    const float3 we = normalize3(f3(cam.aspect * cam.tan_fov * px, cam.tan_fov * py, -1.0f));
    return cam.vx * we.x + cam.vy * we.y + cam.vz * we.z;
}

// BSDF_Flesnel::EvaluateFresnelTerm (bsdf_flesnel.cpp:243-257).
__device__ __forceinline__ float fresnel_dielectric(float wiDotN, float etaI, float etaT)
{
    const float eta = etaI / etaT;
    const float cosThetaTSq = 1.0f - eta * eta * (1.0f - wiDotN * wiDotN);
    if (cosThetaTSq <= 0.0f) return 1.0f;
    const float ci = fabsf(wiDotN), ct = sqrtf(cosThetaTSq);
    const float rs = (etaI * ci - etaT * ct) / (etaI * ci + etaT * ct);
    const float rt = (etaI * ct - etaT * ci) / (etaI * ct + etaT * ci);
    return (rs * rs + rt * rt) * 0.5f;
}

// BSDF_CookTorrance::EvaluateGGX (bsdf_cooktorrance.cpp:187-198).
__device__ __forceinline__ float ggx_d(float3 H, float a)
{
    const float c = H.z;
    if (c <= 0.0f) return 0.0f;
    const float t = 1.0f - c * c;
    const float tanH = t <= 0.0f ? 0.0f : sqrtf(t) / c;
    const float q = a * a + tanH * tanH;
    return (a * a) / (3.14159265358979f * c * c * c * c * q * q);
}

// BSDF_CookTorrance::SampleGGX (bsdf_cooktorrance.cpp:200-225); Math::Eps<float> = 1e-4.
__device__ __forceinline__ float3 ggx_sample(float ua, float ub, float a)
{
    const float eps = 1e-4f;
    const float u0 = (1.0f - eps) * ua + eps;
    const float u1 = (1.0f - 2.0f * eps) * ub + eps;
    const float den = sqrtf(1.0f - (1.0f - a * a) * u0);
    const float cosT = sqrtf(1.0f - u0) / den;
    const float sinT = a * (sqrtf(u0) / den);
    float sp, cp;
    sincosf(3.14159265358979f * (2.0f * u1 - 1.0f), &sp, &cp);
    return f3(sinT * cp, sinT * sp, cosT);
}

// BSDF_CookTorrance::EvaluateFrConductor (bsdf_cooktorrance.cpp:283-291), one channel.
__device__ __forceinline__ float fresnel_conductor(float c, float eta, float k)
{
    const float tmp = (eta * eta + k * k) * (c * c);
    const float rParl2 = (tmp - eta * (2.0f * c) + 1.0f) / (tmp + eta * (2.0f * c) + 1.0f);
    const float tmpF = eta * eta + k * k;
    const float rPerp2 = (tmpF - eta * (2.0f * c) + c * c) / (tmpF + eta * (2.0f * c) + c * c);
    return (rParl2 + rPerp2) * 0.5f;
}

// Samples the BSDF of P at a surface with normal n (shading normal = geometric
// normal: meshes here carry no vertex normals) for the eye-to-light transport
// direction.  Returns false when the path ends; otherwise the world-space
// direction wo and the weight f = fs / pdf (projected solid angle).
__device__ __forceinline__ bool sample_bsdf(const PrimGPU& P, float3 n, float3 wi, float u0, float u1, float u2,
                                            float3& wo, float f[3])
{
    float3 bx, by;
    basis(n, bx, by);
    const float3 lwi = f3(dot3(wi, bx), dot3(wi, by), dot3(wi, n));
    float3 lwo;
    if (P.bsdf == LMGPU_BSDF_DIFFUSE) {
        // bsdf_diffuse.cpp:69-104: one-sided, fs / pdf = R
        if (lwi.z <= 0.0f) return false;
        lwo = cosine_hemisphere(u0, u1);
        if (lwo.z <= 0.0f) return false;
        for (int k = 0; k < 3; k++) f[k] = P.R[k];
    } else if (P.bsdf == LMGPU_BSDF_DIELECTRIC) {
        // bsdf_flesnel.cpp:59-164: reflect with probability Fr, else refract;
        // fs / pdf = R, or R (etaI / etaT)^2 for refraction (EL direction)
        float etaI = P.eta1, etaT = P.eta2;
        if (lwi.z < 0.0f) { const float t = etaI; etaI = etaT; etaT = t; }
        const float Fr = fresnel_dielectric(lwi.z, etaI, etaT);
        float scale = 1.0f;
        if (u2 <= Fr) {
            lwo = f3(-lwi.x, -lwi.y, lwi.z);
        } else {
            const float eta = etaI / etaT;
            const float cosTSq = 1.0f - eta * eta * (1.0f - lwi.z * lwi.z);
            const float cosT = sqrtf(fmaxf(cosTSq, 0.0f)) * (lwi.z > 0.0f ? -1.0f : 1.0f);
            lwo = f3(-eta * lwi.x, -eta * lwi.y, cosT);
            scale = eta * eta;
        }
        for (int k = 0; k < 3; k++) f[k] = P.R[k] * scale;
    } else if (P.bsdf == LMGPU_BSDF_COOK_TORRANCE) {
        // bsdf_cooktorrance.cpp:73-120, GGX; G uses |wo.H| in both terms
        if (lwi.z <= 0.0f) return false;
        const float3 H = ggx_sample(u0, u1, P.roughness);
        const float dih = -dot3(lwi, H);
        lwo = (lwi * -1.0f) - H * (2.0f * dih);
        if (lwo.z <= 0.0f) return false;
        const float3 Hn = normalize3(lwi + lwo);
        const float D = ggx_d(Hn, P.roughness);
        const float woH = fabsf(dot3(lwo, Hn));
        const float G = fminf(1.0f, fminf(2.0f * Hn.z * lwo.z / woH, 2.0f * Hn.z * lwi.z / woH));
        const float pdf = D * Hn.z / (4.0f * dot3(lwo, Hn)) / lwo.z;
        if (!(pdf > 0.0f)) return false;
        const float cih = dot3(lwi, Hn);
        for (int k = 0; k < 3; k++) {
            const float F = fresnel_conductor(cih, P.ct_eta[k], P.ct_k[k]);
            f[k] = (P.R[k] * D * G * F / (4.0f * lwi.z) / lwo.z) / pdf;
        }
    } else {
        return false;  // bsdf::null
    }
    if (f[0] == 0.0f && f[1] == 0.0f && f[2] == 0.0f) return false;
    wo = bx * lwo.x + by * lwo.y + n * lwo.z;
    return true;
}

}  // namespace lmgpu
