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
//   k_film_finalize per-pixel mean and FP64 variance of the mean (scene.cu)
// Sampling differs from the reference only in ways that keep the estimator's
// expectation: raster positions are stratified per pixel (spp jittered
// samples in each pixel instead of W*H*spp uniform positions over the film),
// and random numbers come from Philox keyed by (seed, path, bounce).
#include "accel.cuh"
#include "rng.cuh"
#include "scene.cuh"
#include "bsdf.cuh"

namespace lmgpu {
namespace {

constexpr int kShadeThreads = 256;

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

__device__ __forceinline__ void splat(double* __restrict__ film, double* __restrict__ film_sq, uint32_t pixel,
                                      const float c[3])
{
    for (int k = 0; k < 3; k++) {
        if (c[k] != 0.0f) {
            atomicAdd(&film[3 * (size_t)pixel + k], (double)c[k]);
            atomicAdd(&film_sq[3 * (size_t)pixel + k], (double)c[k] * (double)c[k]);
        }
    }
}

__global__ void __launch_bounds__(kShadeThreads) k_pt_shade(const float4* __restrict__ rays,
                                                            const PathState* __restrict__ state,
                                                            const lmgpu_hit* __restrict__ hits, uint32_t n,
                                                            SceneGPU sc, int max_nv, uint32_t seed,
                                                            double* __restrict__ film, double* __restrict__ film_sq,
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

}  // namespace

int render_pt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream)
{
    const uint32_t W = (uint32_t)sc->cam.width, H = (uint32_t)sc->cam.height;
    const uint64_t npix = (uint64_t)W * H;
    const uint64_t total = npix * prm->spp;
    if (total == 0) return LMGPU_OK;
    int rc = clear_film(sc, npix, stream);
    if (rc) return rc;
    rc = ensure_queues(sc, total < kWave ? total : kWave);
    if (rc) return rc;
    const SceneGPU sg = scene_view(sc);
    for (uint64_t p0 = 0; p0 < total; p0 += kWave) {
        uint32_t n = (uint32_t)((total - p0) < kWave ? (total - p0) : kWave);
        k_pt_generate<<<(n + 255) / 256, 256, 0, stream>>>(sc->cam, p0, n, prm->seed, sc->q_ray[0], sc->q_state[0]);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
        int cur = 0;
        while (n > 0) {
            rc = launch_trace(sc->accel, sc->q_ray[cur], sc->q_hit, n, false, false, stream);
            if (rc) return rc;
            LMGPU_CUDA_TRY(cudaMemsetAsync(sc->q_count, 0, sizeof(uint32_t), stream));
            k_pt_shade<<<(n + kShadeThreads - 1) / kShadeThreads, kShadeThreads, 0, stream>>>(
                sc->q_ray[cur], sc->q_state[cur], sc->q_hit, n, sg, prm->max_num_vertices, prm->seed, sc->film,
                sc->film_sq, sc->q_ray[1 - cur], sc->q_state[1 - cur], sc->q_count);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 2;  // trace + shade
            LMGPU_CUDA_TRY(cudaMemcpyAsync(sc->h_count, sc->q_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
            LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
            n = *sc->h_count;
            cur = 1 - cur;
        }
    }
    return finalize_film(sc, prm->spp, d_image, d_variance, stream);
}

}  // namespace lmgpu
