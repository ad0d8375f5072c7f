// Wavefront path tracers: the GPU forms of renderer::pt, renderer::ptmis and
// renderer::ptdirect.
//
// renderer::pt (src/liblightmetrica/renderer/renderer_pt.cpp:68-231): a path
// starts at the pinhole sensor with throughput 1 (importance / pdf), extends
// by BSDF sampling (fs / pdf), splats throughput * Le whenever it hits the
// front side of an area light (no next-event estimation), applies Russian
// roulette with probability 0.5 after every hit, and stops after
// max_num_vertices vertices or at a surface whose BSDF is null.
//
// renderer::ptmis (renderer_ptmis.cpp:68-305) adds, at every vertex before
// its BSDF sample (the sensor included), one light sample: a light primitive
// chosen uniformly, a triangle by its area CDF, a uniform point on it; the
// contribution fs G V Le / (pdf_light pdf_area) is weighted by the balance
// heuristic pdf_light / (pdf_light + pdf_bsdf) in projected solid angle, and
// BSDF-sampled light hits by pdf_bsdf / (pdf_bsdf + pdf_light), with
// pdf_light = 0 after a specular vertex.  renderer::ptdirect
// (renderer_ptdirect.cpp:72-291) keeps the light samples with weight 1 and
// counts no BSDF-sampled emission at all.  Environment lights are not
// sampled by these two forms (the entry points reject scenes that have one).
//
// BSDFs: bsdf::null, bsdf::diffuse, bsdf::flesnel (dielectric) and
// bsdf::cook_torrance (GGX conductor); lights: light::area on primitives and a
// constant light::env reached by rays that leave the geometry (pt only).
//
// GPU structure, one wave of up to kWave paths at a time:
//   k_pt_generate   camera rays for paths [p0, p0 + n) (sensor_pinhole.cpp:79-90);
//                   ptmis: the sensor's light sample
//   per bounce      k_trace (closest hit, trace.cu) over the compacted queue,
//                   its length read on the device (no host round trip);
//                   k_pt_shade: emission (MIS-weighted for ptmis), roulette,
//                   BSDF sampling, block-aggregated append of surviving paths;
//                   ptmis: the new vertex's light sample as a shadow ray plus
//                   a pending contribution, then k_trace (any hit) over the
//                   shadow rays and k_pt_nee_splat
//   k_pt_flush      each path's own-pixel sum into the film (sum and square:
//                   the reference film squares per-sample sums)
//   k_film_finalize per-pixel mean and FP64 variance of the mean (scene.cu)
// Sampling differs from the reference only in ways that keep the estimator's
// expectation: raster positions are stratified per pixel (spp jittered
// samples in each pixel instead of W*H*spp uniform positions over the film),
// and random numbers come from Philox keyed by (seed, path, bounce).
#include "accel.cuh"
#include "interact.cuh"
#include "rng.cuh"

namespace lmgpu {
namespace {

constexpr int kShadeThreads = 256;

// Estimators of the wavefront tracer.
enum : int { MODE_PT = 0, MODE_PTMIS = 1, MODE_PTDIRECT = 2 };

// PathState.id.w holds, for ptmis, the BSDF pdf of the last sampled
// direction times |cos| at the vertex it left (projected solid angle to
// solid angle at that end; 1 for the pinhole), or -1 after a specular vertex.
__device__ __forceinline__ float light_pdf_proj(const Ctx& C, int prim, float d2, float cos_light)
{
    // pdf_light of reaching `prim` at distance^2 d2, without the previous
    // vertex's cosine: (1 / area) (1 / #lights) d^2 / |cos_light|
    return C.lights.inv_area[C.lights.prim_light[prim]] / (float)C.lights.count * d2 / cos_light;
}

// A light sample from vertex v (Renderer_PTMIS, renderer_ptmis.cpp:131-193):
// the weighted contribution (before visibility) and the light point, or
// false when it is black.
template <bool MIS>
__device__ __forceinline__ bool nee_sample(const Ctx& C, const PV& v, int type, float3 wi, float us, float a0,
                                           float a1, const float thr[3], float c[3], PV& L, float3& ppL)
{
    sample_light(C, us, a0, a1, L);
    ppL = normalize3(L.p - v.p);
    const Spd fsE = eval_dir(C, v, type, wi, ppL, DIR_EL, true);
    if (black(fsE)) return false;
    const Spd fsL = eval_dir(C, L, T_L, zero3(), ppL * -1.0f, DIR_LE, false);
    if (black(fsL)) return false;
    const float G = geometry_term(v, L);
    const float pdfL = 1.0f / (float)C.lights.count;
    const float pdfPL = C.lights.inv_area[C.lights.prim_light[L.prim]];
    float w = 1.0f;
    if (MIS) {
        const float pdfDL = pdfPL / G * pdfL;
        const float pdfB = pdf_dir(C, v, type, wi, ppL);
        w = pdfDL / (pdfDL + pdfB);
    }
    bool any = false;
    for (int k = 0; k < 3; k++) {
        c[k] = thr[k] * fsE.c[k] * G * fsL.c[k] / pdfL / pdfPL * w;
        any = any || (c[k] != 0.0f && c[k] == c[k]);
    }
    return any;
}

template <int MODE>
__global__ void __launch_bounds__(kShadeThreads) k_pt_generate(Ctx C, uint64_t p0, uint32_t n, uint32_t seed,
                                                               float4* __restrict__ rays,
                                                               PathState* __restrict__ state,
                                                               uint32_t* __restrict__ count,
                                                               float* __restrict__ own, float4* __restrict__ nrays,
                                                               float4* __restrict__ nrec,
                                                               uint32_t* __restrict__ npath,
                                                               uint32_t* __restrict__ ncount)
{
    constexpr bool NEE = MODE != MODE_PT;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *count = n;  // every path of the wave starts in the queue
    const CameraGPU& cam = C.cam;
    bool has_nee = false;
    PV v, L;
    float c[3] = {0.0f, 0.0f, 0.0f};
    uint32_t nee_pix = 0;
    if (i < n) {
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
        // pinhole: pdf of the direction = importance, |cos| = 1 (degenerate end)
        s.id = make_uint4((uint32_t)p, (uint32_t)(p >> 32), 1u, __float_as_uint(NEE ? importance(cam, d) : 0.0f));
        // renderer::pt passes no state array: its first shading launch
        // rebuilds this state from the path index (first_state)
        if (state) state[i] = s;
        own[3 * (size_t)i] = 0.0f;
        own[3 * (size_t)i + 1] = 0.0f;
        own[3 * (size_t)i + 2] = 0.0f;
        if (NEE && (C.max_path < 0 || 1 < C.max_path) && (MODE == MODE_PTDIRECT || 2 >= C.min_path)) {
            // the sensor's light sample; it lands where ppL meets the film
            sensor_vertex(C, v);
            const Philox4x32 q = philox4x32_10((uint32_t)p, (uint32_t)(p >> 32), 0u, 1u, seed, kKeyCamera);
            const float one[3] = {1.0f, 1.0f, 1.0f};
            float3 ppL;
            has_nee = nee_sample<MODE == MODE_PTMIS>(C, v, T_E, zero3(), u01(q.v[0]), u01(q.v[1]), u01(q.v[2]),
                                                     one, c, L, ppL);
            if (has_nee) {
                float px, py;
                raster_pos(cam, ppL, px, py);
                nee_pix = pixel_at(cam, px, py);
            }
        }
    }
    if (NEE) append_nee(has_nee, v, L, c, nee_pix, i, nrays, nrec, npath, ncount);
}

// The state k_pt_generate gives path p0 + i of renderer::pt, whose first
// shading launch reads no state array (its queue is still in path order):
// saves writing and reading 32 bytes per path.
__device__ __forceinline__ PathState first_state(const CameraGPU& cam, uint64_t p0, uint32_t i)
{
    const uint64_t p = p0 + i;
    const uint32_t npix = (uint32_t)cam.width * (uint32_t)cam.height;
    PathState s;
    s.thr = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float((uint32_t)(p % npix)));
    s.id = make_uint4((uint32_t)p, (uint32_t)(p >> 32), 1u, __float_as_uint(0.0f));
    return s;
}

template <int MODE>
// 4 blocks of 256 per SM (64 registers): the next-event modes (93-96 registers unbounded)
// measured +5-6 %, renderer::pt (54 registers) unchanged
__global__ void __launch_bounds__(kShadeThreads, 4) k_pt_shade(Ctx C, const float4* __restrict__ rays,
                                                            const PathState* __restrict__ state,
                                                            const lmgpu_hit* __restrict__ hits,
                                                            const uint32_t* __restrict__ d_n, uint64_t p0,
                                                            uint32_t seed, float* __restrict__ own,
                                                            float4* __restrict__ out_rays,
                                                            PathState* __restrict__ out_state,
                                                            uint32_t* __restrict__ out_count,
                                                            float4* __restrict__ nrays, float4* __restrict__ nrec,
                                                            uint32_t* __restrict__ npath,
                                                            uint32_t* __restrict__ ncount)
{
    constexpr bool NEE = MODE != MODE_PT;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *d_n;  // queue length, written by the previous kernel
    bool keep = false, has_nee = false;
    float4 nr0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nr1 = nr0;
    PathState ns;
    PV v, L;
    float c[3] = {0.0f, 0.0f, 0.0f};
    uint32_t pixel = 0, path = 0;
    if (i < n) {
        const lmgpu_hit h = hits[i];
        // state == NULL: renderer::pt's first bounce (first_state)
        const PathState s = (NEE || state) ? state[i] : first_state(C.cam, p0, i);
        pixel = __float_as_uint(s.thr.w);
        const uint64_t p = (uint64_t)s.id.x | ((uint64_t)s.id.y << 32);
        path = (uint32_t)(p - p0);
        float* acc = own + 3 * (size_t)path;
        if (h.prim < 0) {
            // miss: the environment light, if any (scene3.cpp:464-475); the
            // path ends there (renderer_pt.cpp:200-203)
            if (!NEE && C.sc.has_env && (int)s.id.z + 1 >= C.min_path) {
                acc[0] += s.thr.x * C.sc.env_Le[0];
                acc[1] += s.thr.y * C.sc.env_Le[1];
                acc[2] += s.thr.z * C.sc.env_Le[2];
            }
        } else {
            const float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
            const float3 o = f3(r0.x, r0.y, r0.z), d = f3(r1.x, r1.y, r1.z);
            const float* T = C.sc.tris + 9 * (size_t)h.prim;
            const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
            v.p = o + d * h.t;
            v.n = normalize3(cross3(p2 - p1, p3 - p1));
            v.prim = C.sc.tri_prim[h.prim];
            const PrimGPU& P = C.sc.prims[v.prim];
            v.type = (short)bsdf_type(P.bsdf);
            v.degen = 0;
            uint32_t nv = s.id.z;
            const float cos_l = -dot3(d, v.n);
            // min_num_vertices: renderer_pt.cpp:186, renderer_ptmis.cpp:247
            if (MODE != MODE_PTDIRECT && P.is_light && cos_l > 0.0f && (int)nv + 1 >= C.min_path) {
                // throughput * Le(-d) * EvaluatePosition (= 1), renderer_pt.cpp:183-194;
                // ptmis: weight pdf_bsdf / (pdf_bsdf + pdf_light), renderer_ptmis.cpp:246-270
                float w = 1.0f;
                if (MODE == MODE_PTMIS) {
                    const float q = __uint_as_float(s.id.w);
                    w = q < 0.0f ? 1.0f : q / (q + light_pdf_proj(C, v.prim, h.t * h.t, cos_l));
                }
                acc[0] += s.thr.x * P.Le[0] * w;
                acc[1] += s.thr.y * P.Le[1] * w;
                acc[2] += s.thr.z * P.Le[2] * w;
            }
            const Philox4x32 r = philox4x32_10(s.id.x, s.id.y, nv, 0u, seed, kKeyBounce);
            // Russian roulette, probability 0.5 (renderer_pt.cpp:207-216)
            if (u01(r.v[3]) <= 0.5f) {
                nv++;
                const bool more = C.max_path < 0 || (int)nv < C.max_path;
                const float thr[3] = {2.0f * s.thr.x, 2.0f * s.thr.y, 2.0f * s.thr.z};
                const float3 wi = d * -1.0f;
                // renderer::ptmis samples a light only for paths of at least
                // min_num_vertices (renderer_ptmis.cpp:132); ptdirect ignores it
                if (more && NEE && (MODE == MODE_PTDIRECT || (int)nv + 1 >= C.min_path)) {
                    const Philox4x32 q = philox4x32_10(s.id.x, s.id.y, nv, 1u, seed, kKeyBounce);
                    float3 ppL;
                    has_nee = nee_sample<MODE == MODE_PTMIS>(C, v, v.type, wi, u01(q.v[0]), u01(q.v[1]),
                                                             u01(q.v[2]), thr, c, L, ppL);
                }
                float3 wo;
                float f[3];
                float q_next = 0.0f;
                bool ok = false;
                if (more) {
                    if (NEE) {
                        ok = sample_dir(C, v, wi, u01(r.v[0]), u01(r.v[1]), u01(r.v[2]), wo);
                        if (ok) {
                            const Spd fs = eval_dir(C, v, v.type, wi, wo, DIR_EL, false);
                            const float pdfD = pdf_dir(C, v, v.type, wi, wo);
                            ok = !black(fs) && pdfD > 0.0f;
                            for (int k = 0; k < 3; k++) f[k] = fs.c[k] / pdfD;
                            q_next = delta_dir(C, v, v.type) ? -1.0f : pdfD * fabsf(dot3(v.n, wo));
                        }
                    } else {
                        ok = sample_bsdf(P, v.n, wi, u01(r.v[0]), u01(r.v[1]), u01(r.v[2]), wo, f);
                    }
                }
                if (ok) {
                    keep = true;
                    nr0 = make_float4(v.p.x, v.p.y, v.p.z, 1e-4f);
                    nr1 = make_float4(wo.x, wo.y, wo.z, FLT_MAX);
                    ns.thr = make_float4(thr[0] * f[0], thr[1] * f[1], thr[2] * f[2], s.thr.w);
                    ns.id = make_uint4(s.id.x, s.id.y, nv, __float_as_uint(q_next));
                }
            }
        }
    }
    if (NEE) append_nee(has_nee, v, L, c, pixel, path, nrays, nrec, npath, ncount);
    // block-aggregated append to the next queue: one global atomic per block
    // (one per warp serialised on the queue counter)
    __shared__ uint32_t s_warp[kShadeThreads / 32];
    __shared__ uint32_t s_base;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0u) s_warp[warp] = (uint32_t)__popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int k = 0; k < kShadeThreads / 32; k++) {
            const uint32_t cw = s_warp[k];
            s_warp[k] = tot;
            tot += cw;
        }
        s_base = tot ? atomicAdd(out_count, tot) : 0u;
    }
    __syncthreads();
    if (keep) {
        const uint32_t o = s_base + s_warp[warp] + __popc(m & ((1u << lane) - 1u));
        out_rays[2 * o] = nr0;
        out_rays[2 * o + 1] = nr1;
        out_state[o] = ns;
    }
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

// Unoccluded light samples: into the path's own-pixel sum, or (the sensor's
// light samples that land elsewhere) into the film of other samples' splats.
__global__ void k_pt_nee_splat(uint64_t p0, uint32_t npix, const uint32_t* __restrict__ d_n,
                               const float4* __restrict__ rec, const uint32_t* __restrict__ rec_path,
                               const lmgpu_hit* __restrict__ hits, float* __restrict__ own,
                               double* __restrict__ film_x, double* __restrict__ film_x_sq)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= *d_n || hits[q].prim >= 0) return;
    const float4 r = rec[q];
    const uint32_t path = rec_path[q];
    const uint32_t pix = __float_as_uint(r.w);
    const float c[3] = {r.x, r.y, r.z};
    if (pix == (uint32_t)((p0 + path) % npix)) {
        for (int k = 0; k < 3; k++) atomicAdd(&own[3 * (size_t)path + k], c[k]);
    } else {
        splat_px(film_x, film_x_sq, pix, c);
    }
}

__global__ void k_pt_flush(uint64_t p0, uint32_t npix, uint32_t n, const float* __restrict__ own,
                           double* __restrict__ film, double* __restrict__ film_sq)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c[3] = {own[3 * (size_t)i], own[3 * (size_t)i + 1], own[3 * (size_t)i + 2]};
    splat_px(film, film_sq, (uint32_t)((p0 + i) % npix), c);
}

}  // namespace

int render_pt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream,
              int mode)
{
    const bool nee = mode != MODE_PT;
    const char* name = mode == MODE_PTMIS ? "lmgpu_render_ptmis" : "lmgpu_render_ptdirect";
    const uint32_t W = (uint32_t)sc->cam.width, H = (uint32_t)sc->cam.height;
    const uint64_t npix = (uint64_t)W * H;
    const uint64_t total = npix * prm->spp;
    if (total == 0) return LMGPU_OK;
    if (nee && sc->lights.count == 0) {
        set_error(std::string(name) + ": the scene has no area light");
        return LMGPU_ERR_INVALID;
    }
    if (nee && sc->has_env) {
        set_error(std::string(name) + ": environment lights are not sampled by this renderer");
        return LMGPU_ERR_INVALID;
    }
    int rc = clear_film(sc, npix, stream);
    if (rc) return rc;
    rc = ensure_queues(sc, total < kWave ? total : kWave);
    if (rc) return rc;
    Ctx C;
    C.sc = scene_view(sc);
    C.lights = sc->lights;
    C.cam = sc->cam;
    C.max_v = 0;
    C.max_path = prm->max_num_vertices;
    C.min_path = prm->min_num_vertices;
    const uint32_t np = (uint32_t)npix;
    // Queue lengths live on the device (q_count: [0], [1] path queues, [2]
    // pending light samples), so a wave's bounces are queued without host
    // round trips.  With max_num_vertices bounded, the queue is empty after
    // max_num_vertices - 1 bounces; otherwise the host checks every
    // kCheckEvery bounces.
    constexpr int kCheckEvery = 8;
    constexpr int kMaxBounces = 1 << 16;
    const bool bounded = prm->max_num_vertices >= 0;
    const int maxb = bounded ? (prm->max_num_vertices > 1 ? prm->max_num_vertices - 1 : 0) : kMaxBounces;
    auto gen = mode == MODE_PTMIS ? k_pt_generate<MODE_PTMIS>
                                  : (mode == MODE_PTDIRECT ? k_pt_generate<MODE_PTDIRECT> : k_pt_generate<MODE_PT>);
    auto shade = mode == MODE_PTMIS ? k_pt_shade<MODE_PTMIS>
                                    : (mode == MODE_PTDIRECT ? k_pt_shade<MODE_PTDIRECT> : k_pt_shade<MODE_PT>);
    uint32_t* cnt = sc->q_count;
    for (uint64_t p0 = 0; p0 < total; p0 += kWave) {
        const uint32_t n_wave = (uint32_t)((total - p0) < kWave ? (total - p0) : kWave);
        const unsigned gblocks = (n_wave + kShadeThreads - 1) / kShadeThreads;
        LMGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, 4 * sizeof(uint32_t), stream));
        // renderer::pt's first bounce rebuilds its states (first_state)
        PathState* const first = nee ? sc->q_state[0] : nullptr;
        gen<<<gblocks, kShadeThreads, 0, stream>>>(C, p0, n_wave, prm->seed, sc->q_ray[0], first, cnt,
                                                   sc->q_own, sc->q_nray, sc->q_nrec, sc->q_npath, cnt + 2);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
        int cur = 0;
        for (int b = 0;; b++) {
            if (nee) {
                // the light samples of the previous kernel
                rc = launch_trace_dn(sc->accel, sc->q_nray, sc->q_nhit, cnt + 2, n_wave, true, stream, sc->probe);
                if (rc) return rc;
                k_pt_nee_splat<<<gblocks, kShadeThreads, 0, stream>>>(p0, np, cnt + 2, sc->q_nrec, sc->q_npath,
                                                                      sc->q_nhit, sc->q_own, sc->film_x,
                                                                      sc->film_x_sq);
                LMGPU_CUDA_TRY(cudaGetLastError());
                sc->launches += 2;
            }
            if (b >= maxb) break;
            rc = launch_trace_dn(sc->accel, sc->q_ray[cur], sc->q_hit, cnt + cur, n_wave, false, stream, sc->probe);
            if (rc) return rc;
            LMGPU_CUDA_TRY(cudaMemsetAsync(cnt + (1 - cur), 0, sizeof(uint32_t), stream));
            LMGPU_CUDA_TRY(cudaMemsetAsync(cnt + 2, 0, sizeof(uint32_t), stream));
            shade<<<gblocks, kShadeThreads, 0, stream>>>(C, sc->q_ray[cur], b == 0 ? first : sc->q_state[cur],
                                                         sc->q_hit, cnt + cur, p0, prm->seed, sc->q_own,
                                                         sc->q_ray[1 - cur], sc->q_state[1 - cur], cnt + (1 - cur),
                                                         sc->q_nray, sc->q_nrec, sc->q_npath, cnt + 2);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 2;  // trace + shade
            cur = 1 - cur;
            if (!bounded && (b + 1) % kCheckEvery == 0) {
                LMGPU_CUDA_TRY(
                    cudaMemcpyAsync(sc->h_count, cnt, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
                LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
                if (sc->h_count[cur] == 0 && sc->h_count[2] == 0) break;
            }
        }
        k_pt_flush<<<gblocks, kShadeThreads, 0, stream>>>(p0, np, n_wave, sc->q_own, sc->film, sc->film_sq);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
    }
    return finalize_film(sc, prm->spp, d_image, d_variance, stream);
}

}  // namespace lmgpu
