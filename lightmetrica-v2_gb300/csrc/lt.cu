// Light tracing with a sensor connection at every vertex: the GPU form of
// renderer::ltdirect (src/liblightmetrica/renderer/renderer_ltdirect.cpp:72-279).
//
// A light path starts on an area light: a light primitive chosen uniformly
// (Scene3::SampleEmitter, scene3.cpp:506-539), a triangle by its area CDF and
// a uniform point on it, the emission direction drawn from the same 2D
// sample as the position (light_area.cpp:73-80), throughput
// EvaluatePosition / pdf_position / pdf_light = #lights x area (:95-100).
// At every vertex while the path has fewer than max_num_vertices vertices
// (:112-116):
//   sensor connection  the pinhole position; contribution
//                      throughput fs(wi -> sensor) G V We / (pdf_E pdf_PE),
//                      pdf_E = pdf_PE = 1, splatted where the connection
//                      meets the film (:118-168); a visibility ray each
//   next direction     the emission direction at the light, BSDF sampling
//                      elsewhere; throughput *= fs / pdf (:170-205)
//   intersection       the path ends on a miss (:207-219), else Russian
//                      roulette with probability 0.5 (:223-235)
// Every splat lands at a pixel the path does not own, so the film is the
// "other samples" accumulation of the renderers' films: image = sum /
// (light paths per pixel), the reference's W H / N scale (film_hdr.cpp:282-293).
// Scenes with light::env are rejected (only area lights start paths here).
//
// GPU structure, one wave of up to kLtWave paths at a time:
//   k_lt_generate   the light vertex: its sensor connection (a shadow ray and
//                   a pending splat) and the first extension ray
//   per bounce      k_trace (closest hit) over the compacted path queue, any
//                   hit over the pending connections and k_lt_splat (queue
//                   lengths read on the device, no host round trip), then
//                   k_lt_shade: roulette, the vertex's sensor connection,
//                   BSDF sampling, warp-aggregated append
#include "accel.cuh"
#include "interact.cuh"
#include "rng.cuh"

namespace lmgpu {
namespace {

constexpr int kLtThreads = 256;
constexpr uint32_t kLtWave = 1u << 22;
constexpr uint32_t kKeyLightPath = 0x4C505448u;  // light selection, position + emission direction
constexpr uint32_t kKeyLightStep = 0x4C535450u;  // BSDF sample + roulette per light-path vertex

// The sensor connection of light-path vertex v reached along -wi (type: its
// interaction): contribution before visibility and the pixel; false if black.
__device__ __forceinline__ bool sensor_connect(const Ctx& C, const PV& v, int type, float3 wi, const float thr[3],
                                               float c[3], uint32_t& pix, PV& E)
{
    sensor_vertex(C, E);
    const float3 ppE = normalize3(E.p - v.p);
    const Spd fsL = eval_dir(C, v, type, wi, ppE, DIR_LE, true);
    if (black(fsL)) return false;
    const float3 wE = ppE * -1.0f;
    float rx, ry;
    if (!raster_pos(C.cam, wE, rx, ry)) return false;
    const float fsE = importance(C.cam, wE);
    const float G = geometry_term(v, E);
    bool any = false;
    for (int k = 0; k < 3; k++) {
        c[k] = thr[k] * fsL.c[k] * G * fsE;
        any = any || (c[k] != 0.0f && c[k] == c[k]);
    }
    pix = pixel_at(C.cam, rx, ry);
    return any;
}

// Append of a path to the next queue, one queue-counter atomic per block;
// every thread of the block calls it (block_append_slot).
__device__ __forceinline__ void append_path(bool keep, float4 r0, float4 r1, const PathState& s,
                                            float4* __restrict__ rays, PathState* __restrict__ state,
                                            uint32_t* __restrict__ count)
{
    const uint32_t o = block_append_slot<kLtThreads / 32>(keep, count);
    if (keep) {
        rays[2 * o] = r0;
        rays[2 * o + 1] = r1;
        state[o] = s;
    }
}

__global__ void __launch_bounds__(kLtThreads) k_lt_generate(Ctx C, uint64_t p0, uint32_t n, uint32_t seed,
                                                            float4* __restrict__ rays, PathState* __restrict__ state,
                                                            uint32_t* __restrict__ count, float4* __restrict__ nrays,
                                                            float4* __restrict__ nrec, uint32_t* __restrict__ npath,
                                                            uint32_t* __restrict__ ncount)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false, has_nee = false;
    PV v, E;
    float c[3] = {0.0f, 0.0f, 0.0f};
    uint32_t pix = 0;
    float4 r0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), r1 = r0;
    PathState s;
    if (i < n) {
        const uint64_t p = p0 + i;
        const Philox4x32 r = philox4x32_10((uint32_t)p, (uint32_t)(p >> 32), 0u, 0u, seed, kKeyLightPath);
        const float a0 = u01(r.v[1]), a1 = u01(r.v[2]);
        sample_light(C, u01(r.v[0]), a0, a1, v);
        const float t0 = (float)C.lights.count / C.lights.inv_area[C.lights.prim_light[v.prim]];
        float thr[3] = {t0, t0, t0};
        if (C.max_path < 0 || 1 < C.max_path) {
            has_nee = sensor_connect(C, v, T_L, zero3(), thr, c, pix, E);
            const float3 l = cosine_hemisphere(a0, a1);
            float3 b, cc;
            basis(v.n, b, cc);
            const float3 wo = b * l.x + cc * l.y + v.n * l.z;
            const Spd fs = eval_dir(C, v, T_L, zero3(), wo, DIR_LE, false);
            const float pdfD = pdf_dir(C, v, T_L, zero3(), wo);
            if (!black(fs) && pdfD > 0.0f) {
                keep = true;
                r0 = make_float4(v.p.x, v.p.y, v.p.z, 1e-4f);
                r1 = make_float4(wo.x, wo.y, wo.z, FLT_MAX);
                s.thr = make_float4(thr[0] * fs.c[0] / pdfD, thr[1] * fs.c[1] / pdfD, thr[2] * fs.c[2] / pdfD, 0.0f);
                s.id = make_uint4((uint32_t)p, (uint32_t)(p >> 32), 1u, 0u);
            }
        }
    }
    append_nee(has_nee, v, E, c, pix, i, nrays, nrec, npath, ncount);
    append_path(keep, r0, r1, s, rays, state, count);
}

// 4 blocks of 256 per SM (64 registers): +2.6 % over the unbounded 91-register build
__global__ void __launch_bounds__(kLtThreads, 4) k_lt_shade(Ctx C, const float4* __restrict__ rays,
                                                         const PathState* __restrict__ state,
                                                         const lmgpu_hit* __restrict__ hits,
                                                         const uint32_t* __restrict__ d_n, uint64_t p0,
                                                         uint32_t seed, float4* __restrict__ out_rays,
                                                         PathState* __restrict__ out_state,
                                                         uint32_t* __restrict__ out_count, float4* __restrict__ nrays,
                                                         float4* __restrict__ nrec, uint32_t* __restrict__ npath,
                                                         uint32_t* __restrict__ ncount)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *d_n;  // queue length, written by the previous kernel
    bool keep = false, has_nee = false;
    PV v, E;
    float c[3] = {0.0f, 0.0f, 0.0f};
    uint32_t pix = 0, path = 0;
    float4 r0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), r1 = r0;
    PathState ns;
    if (i < n) {
        const lmgpu_hit h = hits[i];
        const PathState s = state[i];
        const uint64_t p = (uint64_t)s.id.x | ((uint64_t)s.id.y << 32);
        path = (uint32_t)(p - p0);
        const uint32_t nv = s.id.z + 1u;
        const Philox4x32 r = philox4x32_10(s.id.x, s.id.y, nv, 0u, seed, kKeyLightStep);
        if (h.prim >= 0 && u01(r.v[3]) <= 0.5f) {
            const float4 q0 = rays[2 * i], q1 = rays[2 * i + 1];
            const float3 o = f3(q0.x, q0.y, q0.z), d = f3(q1.x, q1.y, q1.z);
            const float* T = C.sc.tris + 9 * (size_t)h.prim;
            const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
            v.p = o + d * h.t;
            v.n = normalize3(cross3(p2 - p1, p3 - p1));
            v.prim = C.sc.tri_prim[h.prim];
            v.type = (short)bsdf_type(C.sc.prims[v.prim].bsdf);
            v.degen = 0;
            const float thr[3] = {2.0f * s.thr.x, 2.0f * s.thr.y, 2.0f * s.thr.z};
            const float3 wi = d * -1.0f;
            if (C.max_path < 0 || (int)nv < C.max_path) {
                has_nee = sensor_connect(C, v, v.type, wi, thr, c, pix, E);
                float3 wo;
                if (sample_dir(C, v, wi, u01(r.v[0]), u01(r.v[1]), u01(r.v[2]), wo)) {
                    const Spd fs = eval_dir(C, v, v.type, wi, wo, DIR_LE, false);
                    const float pdfD = pdf_dir(C, v, v.type, wi, wo);
                    if (!black(fs) && pdfD > 0.0f) {
                        keep = true;
                        r0 = make_float4(v.p.x, v.p.y, v.p.z, 1e-4f);
                        r1 = make_float4(wo.x, wo.y, wo.z, FLT_MAX);
                        ns.thr = make_float4(thr[0] * fs.c[0] / pdfD, thr[1] * fs.c[1] / pdfD,
                                             thr[2] * fs.c[2] / pdfD, 0.0f);
                        ns.id = make_uint4(s.id.x, s.id.y, nv, 0u);
                    }
                }
            }
        }
    }
    append_nee(has_nee, v, E, c, pix, path, nrays, nrec, npath, ncount);
    append_path(keep, r0, r1, ns, out_rays, out_state, out_count);
}

// Unoccluded sensor connections into the film of other samples' splats.
__global__ void k_lt_splat(const uint32_t* __restrict__ d_n, const float4* __restrict__ rec,
                           const lmgpu_hit* __restrict__ hits, double* __restrict__ film_x,
                           double* __restrict__ film_x_sq)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= *d_n || hits[q].prim >= 0) return;
    const float4 r = rec[q];
    const size_t pix = __float_as_uint(r.w);
    const float c[3] = {r.x, r.y, r.z};
    for (int k = 0; k < 3; k++) {
        if (c[k] != 0.0f) {
            atomicAdd(&film_x[3 * pix + k], (double)c[k]);
            atomicAdd(&film_x_sq[3 * pix + k], (double)c[k] * (double)c[k]);
        }
    }
}

}  // namespace

int render_ltdirect(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance,
                    cudaStream_t stream)
{
    const char* name = "lmgpu_render_ltdirect";
    const uint64_t npix = (uint64_t)sc->cam.width * sc->cam.height;
    const uint64_t total = npix * prm->spp;
    if (total == 0) return LMGPU_OK;
    if (sc->lights.count == 0) {
        set_error(std::string(name) + ": the scene has no area light");
        return LMGPU_ERR_INVALID;
    }
    if (sc->has_env) {
        set_error(std::string(name) + ": environment lights are not sampled by this renderer");
        return LMGPU_ERR_INVALID;
    }
    int rc = clear_film(sc, npix, stream);
    if (rc) return rc;
    rc = ensure_queues(sc, total < kLtWave ? total : kLtWave);
    if (rc) return rc;
    Ctx C;
    C.sc = scene_view(sc);
    C.lights = sc->lights;
    C.cam = sc->cam;
    C.max_v = 0;
    C.max_path = prm->max_num_vertices;
    // Queue lengths on the device (q_count: [0], [1] path queues, [2]
    // pending sensor connections): a wave's bounces are queued without host
    // round trips; with max_num_vertices bounded the queue is empty after
    // max_num_vertices - 1 bounces, otherwise the host checks every
    // kCheckEvery bounces.
    constexpr int kCheckEvery = 8;
    constexpr int kMaxBounces = 1 << 16;
    const bool bounded = prm->max_num_vertices >= 0;
    const int maxb = bounded ? (prm->max_num_vertices > 1 ? prm->max_num_vertices - 1 : 0) : kMaxBounces;
    uint32_t* cnt = sc->q_count;
    for (uint64_t p0 = 0; p0 < total; p0 += kLtWave) {
        const uint32_t n_wave = (uint32_t)((total - p0) < kLtWave ? (total - p0) : kLtWave);
        const unsigned gblocks = (n_wave + kLtThreads - 1) / kLtThreads;
        LMGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, 4 * sizeof(uint32_t), stream));
        k_lt_generate<<<gblocks, kLtThreads, 0, stream>>>(C, p0, n_wave, prm->seed, sc->q_ray[0], sc->q_state[0],
                                                          cnt, sc->q_nray, sc->q_nrec, sc->q_npath, cnt + 2);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
        int cur = 0;
        for (int b = 0;; b++) {
            // the sensor connections of the previous kernel
            rc = launch_trace_dn(sc->accel, sc->q_nray, sc->q_nhit, cnt + 2, n_wave, true, stream, sc->probe);
            if (rc) return rc;
            k_lt_splat<<<gblocks, kLtThreads, 0, stream>>>(cnt + 2, sc->q_nrec, sc->q_nhit, sc->film_x,
                                                           sc->film_x_sq);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 2;
            if (b >= maxb) break;
            rc = launch_trace_dn(sc->accel, sc->q_ray[cur], sc->q_hit, cnt + cur, n_wave, false, stream, sc->probe);
            if (rc) return rc;
            LMGPU_CUDA_TRY(cudaMemsetAsync(cnt + (1 - cur), 0, sizeof(uint32_t), stream));
            LMGPU_CUDA_TRY(cudaMemsetAsync(cnt + 2, 0, sizeof(uint32_t), stream));
            k_lt_shade<<<gblocks, kLtThreads, 0, stream>>>(C, sc->q_ray[cur], sc->q_state[cur], sc->q_hit, cnt + cur,
                                                           p0, prm->seed, sc->q_ray[1 - cur], sc->q_state[1 - cur],
                                                           cnt + (1 - cur), sc->q_nray, sc->q_nrec, sc->q_npath,
                                                           cnt + 2);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 2;
            cur = 1 - cur;
            if (!bounded && (b + 1) % kCheckEvery == 0) {
                LMGPU_CUDA_TRY(
                    cudaMemcpyAsync(sc->h_count, cnt, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
                LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
                if (sc->h_count[cur] == 0 && sc->h_count[2] == 0) break;
            }
        }
    }
    // every splat is another sample's: n_x = all light paths
    return finalize_film_nx(sc, prm->spp, (double)total, d_image, d_variance, stream);
}

}  // namespace lmgpu
