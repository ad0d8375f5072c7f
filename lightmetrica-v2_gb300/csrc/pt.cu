// Wavefront path tracer: the GPU form of renderer::pt.
//
// Reference behaviour (src/liblightmetrica/renderer/renderer_pt.cpp:68-231):
// a path starts at the pinhole sensor with throughput 1 (importance / pdf),
// extends by BSDF sampling (fs / pdf), splats throughput * Le whenever it
// hits the front side of an area light (no next-event estimation), applies
// Russian roulette with probability 0.5 after every hit, and stops after
// max_num_vertices vertices or at a surface whose BSDF is null.
//
// BSDFs: bsdf::null, bsdf::diffuse, bsdf::flesnel (dielectric) and
// bsdf::cook_torrance (GGX conductor); lights: light::area on primitives and a
// constant light::env reached by rays that leave the geometry.
//
// GPU structure, one wave of up to kWave paths at a time:
//   k_pt_generate   camera rays for paths [p0, p0 + n) (sensor_pinhole.cpp:79-90)
//   k_trace         closest hit for the queue (trace.cu)
//   k_pt_shade      emission splat, roulette, diffuse sampling
//                   (bsdf_diffuse.cpp:69-104, sampler.h:44-67); surviving
//                   paths are appended to the next queue (warp-aggregated
//                   atomics, so queues stay compact)
//   k_pt_finalize   per-pixel mean and FP64 variance of the mean
// Sampling differs from the reference only in ways that keep the estimator's
// expectation: raster positions are stratified per pixel (spp jittered
// samples in each pixel instead of W*H*spp uniform positions over the film),
// and random numbers come from Philox keyed by (seed, path, bounce).
#include "accel.cuh"
#include "rng.cuh"
#include "scene.cuh"

namespace lmgpu {
namespace {

constexpr int kShadeThreads = 256;

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

__global__ void k_pt_generate(CameraGPU cam, uint64_t p0, uint32_t n, uint32_t seed, float4* __restrict__ rays,
                              PathState* __restrict__ state)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t p = p0 + i;
    const uint32_t npix = (uint32_t)cam.width * (uint32_t)cam.height;
    const uint32_t pixel = (uint32_t)(p % npix);
    const uint32_t x = pixel % (uint32_t)cam.width, y = pixel / (uint32_t)cam.width;
    const Philox4x32 r = philox4x32_10((uint32_t)p, (uint32_t)(p >> 32), 0u, 0u, seed, kKeyCamera);
    const float rx = ((float)x + u01(r.v[0])) / (float)cam.width;
    const float ry = ((float)y + u01(r.v[1])) / (float)cam.height;
    const float3 d = camera_dir(cam, rx, ry);
    rays[2 * i] = make_float4(cam.eye.x, cam.eye.y, cam.eye.z, 1e-4f);
    rays[2 * i + 1] = make_float4(d.x, d.y, d.z, FLT_MAX);
    PathState s;
    s.thr = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(pixel));
    s.id = make_uint4((uint32_t)p, (uint32_t)(p >> 32), 1u, 0u);
    state[i] = s;
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

__device__ __forceinline__ void splat(float* __restrict__ film, double* __restrict__ film_sq, uint32_t pixel,
                                      const float c[3])
{
    for (int k = 0; k < 3; k++) {
        if (c[k] != 0.0f) {
            atomicAdd(&film[3 * (size_t)pixel + k], c[k]);
            atomicAdd(&film_sq[3 * (size_t)pixel + k], (double)c[k] * (double)c[k]);
        }
    }
}

__global__ void __launch_bounds__(kShadeThreads) k_pt_shade(const float4* __restrict__ rays,
                                                            const PathState* __restrict__ state,
                                                            const lmgpu_hit* __restrict__ hits, uint32_t n,
                                                            SceneGPU sc, int max_nv, uint32_t seed,
                                                            float* __restrict__ film, double* __restrict__ film_sq,
                                                            float4* __restrict__ out_rays,
                                                            PathState* __restrict__ out_state,
                                                            uint32_t* __restrict__ out_count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    float4 nr0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nr1 = nr0;
    PathState ns;
    if (i < n) {
        const lmgpu_hit h = hits[i];
        const PathState s = state[i];
        const uint32_t pixel = __float_as_uint(s.thr.w);
        if (h.prim < 0) {
            // miss: the environment light, if any (scene3.cpp:464-475); the
            // path ends there (renderer_pt.cpp:200-203)
            if (sc.has_env) {
                const float c[3] = {s.thr.x * sc.env_Le[0], s.thr.y * sc.env_Le[1], s.thr.z * sc.env_Le[2]};
                splat(film, film_sq, pixel, c);
            }
        } else {
            const float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
            const float3 o = f3(r0.x, r0.y, r0.z), d = f3(r1.x, r1.y, r1.z);
            const float* T = sc.tris + 9 * (size_t)h.prim;
            const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
            const float3 gn = normalize3(cross3(p2 - p1, p3 - p1));
            const PrimGPU P = sc.prims[sc.tri_prim[h.prim]];
            const float3 pos = o + d * h.t;
            uint32_t nv = s.id.z;
            if (P.is_light && -dot3(d, gn) > 0.0f) {
                // throughput * Le(-d) * EvaluatePosition (= 1), renderer_pt.cpp:183-194
                const float c[3] = {s.thr.x * P.Le[0], s.thr.y * P.Le[1], s.thr.z * P.Le[2]};
                splat(film, film_sq, pixel, c);
            }
            const Philox4x32 r = philox4x32_10(s.id.x, s.id.y, nv, 0u, seed, kKeyBounce);
            // Russian roulette, probability 0.5 (renderer_pt.cpp:207-216)
            if (u01(r.v[3]) <= 0.5f) {
                nv++;
                const bool more = max_nv < 0 || (int)nv < max_nv;
                float3 wo;
                float f[3];
                if (more && sample_bsdf(P, gn, d * -1.0f, u01(r.v[0]), u01(r.v[1]), u01(r.v[2]), wo, f)) {
                    keep = true;
                    nr0 = make_float4(pos.x, pos.y, pos.z, 1e-4f);
                    nr1 = make_float4(wo.x, wo.y, wo.z, FLT_MAX);
                    ns.thr = make_float4(2.0f * s.thr.x * f[0], 2.0f * s.thr.y * f[1], 2.0f * s.thr.z * f[2],
                                         s.thr.w);
                    ns.id = make_uint4(s.id.x, s.id.y, nv, 0u);
                }
            }
        }
    }
    // warp-aggregated append to the next queue
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (m == 0u) return;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(out_count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (keep) {
        const uint32_t o = base + __popc(m & ((1u << lane) - 1u));
        out_rays[2 * o] = nr0;
        out_rays[2 * o + 1] = nr1;
        out_state[o] = ns;
    }
}

__global__ void k_pt_finalize(const float* __restrict__ film, const double* __restrict__ film_sq, uint32_t n3,
                              double spp, float* __restrict__ image, float* __restrict__ variance)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const double mean = (double)film[i] / spp;
    image[i] = (float)mean;
    if (variance) {
        const double v = (film_sq[i] / spp - mean * mean) / spp;
        variance[i] = (float)(v > 0.0 ? v : 0.0);
    }
}

}  // namespace

int render_pt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream)
{
    const uint32_t W = (uint32_t)sc->cam.width, H = (uint32_t)sc->cam.height;
    const uint64_t npix = (uint64_t)W * H;
    const uint64_t total = npix * prm->spp;
    if (total == 0) return LMGPU_OK;
    int rc = ensure_film(sc, npix);
    if (rc) return rc;
    rc = ensure_queues(sc, total < kWave ? total : kWave);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemsetAsync(sc->film, 0, sizeof(float) * 3 * npix, stream));
    LMGPU_CUDA_TRY(cudaMemsetAsync(sc->film_sq, 0, sizeof(double) * 3 * npix, stream));
    const SceneGPU sg = scene_view(sc);
    for (uint64_t p0 = 0; p0 < total; p0 += kWave) {
        uint32_t n = (uint32_t)((total - p0) < kWave ? (total - p0) : kWave);
        k_pt_generate<<<(n + 255) / 256, 256, 0, stream>>>(sc->cam, p0, n, prm->seed, sc->q_ray[0], sc->q_state[0]);
        LMGPU_CUDA_TRY(cudaGetLastError());
        int cur = 0;
        while (n > 0) {
            rc = launch_trace(sc->accel, sc->q_ray[cur], sc->q_hit, n, false, false, stream);
            if (rc) return rc;
            LMGPU_CUDA_TRY(cudaMemsetAsync(sc->q_count, 0, sizeof(uint32_t), stream));
            k_pt_shade<<<(n + kShadeThreads - 1) / kShadeThreads, kShadeThreads, 0, stream>>>(
                sc->q_ray[cur], sc->q_state[cur], sc->q_hit, n, sg, prm->max_num_vertices, prm->seed, sc->film,
                sc->film_sq, sc->q_ray[1 - cur], sc->q_state[1 - cur], sc->q_count);
            LMGPU_CUDA_TRY(cudaGetLastError());
            LMGPU_CUDA_TRY(cudaMemcpyAsync(sc->h_count, sc->q_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
            LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
            n = *sc->h_count;
            cur = 1 - cur;
        }
    }
    const uint32_t n3 = (uint32_t)(3 * npix);
    k_pt_finalize<<<(n3 + 255) / 256, 256, 0, stream>>>(sc->film, sc->film_sq, n3, (double)prm->spp, d_image,
                                                       d_variance);
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

}  // namespace lmgpu
