// Guided path tracing: renderer::pt's estimator with the direction at every
// diffuse vertex drawn from a one-sample MIS mixture of BSDF sampling
// (probability alpha) and the learned von Mises-Fisher mixture of the
// guiding network (guide.cu), trained online between passes on radiance
// samples the tracer itself produces.
//
// Estimator: at a diffuse vertex the direction w comes from the BSDF (cosine)
// with probability alpha, else from the network's mixture q; its weight is
// f cos / (alpha cos / pi + (1 - alpha) q(w)), so every pass is unbiased for
// whatever network it used.  Other BSDFs sample as in renderer::pt.  Each
// pass is one sample per pixel.  Russian roulette is renderer::pt's (survival
// 0.5, rr_mode 0) or survival min(1, max throughput) (rr_mode 1), which keeps
// path weights near 1 where guided weights would otherwise compound (up to
// 1 / alpha per vertex); both are unbiased.  A wave holds as many passes as fit in 2^21
// paths (the network is trained after each wave); the film averages all
// passes.
//
// Training data: every guided vertex records its query (position, normal,
// outgoing direction), the sampled direction, the mixture pdf and the
// throughput after the vertex; emission met later along the path is divided
// by that throughput and summed into the vertex's incident radiance L.
// After a pass, vertices with L > 0 become samples of weight
// luminance(L) cos / pdf (target proportional to L cos); the network takes
// Adam steps on them (at most max_steps_per_pass minibatches).
//
// Per bounce: k_trace (closest hit), k_gd_shade (emission into the film and
// the vertex records, roulette, non-diffuse sampling, diffuse queries),
// guide forward on the queries, k_gd_sample (mixture sampling, records).
#include "accel.cuh"
#include "bsdf.cuh"
#include "guide_api.cuh"
#include "guide_net.cuh"
#include "rng.cuh"
#include "scene.cuh"

#include <vector>

namespace lmgpu {
namespace {

// Paths per wave of the guided tracer: whole passes, trained between waves.
constexpr uint64_t kGuidedWave = 1ull << 21;

using namespace guide;

constexpr int kGdThreads = 256;
constexpr int kMaxRec = 8;                  // guided vertices recorded per path
constexpr uint32_t kKeyGuide = 0x47554944u;  // mixture-sampling random numbers

struct GuideRec {
    float4 x;     // position, pdf of the sampled direction
    float4 n;     // normal, -
    float4 wo;    // outgoing direction, -
    float4 wi;    // sampled direction, -
    float4 inv_t; // 1 / throughput after the vertex (rgb), -
    float4 L;     // incident radiance gathered along wi (rgb), -
};

struct Wave {
    uint64_t p0;
    uint32_t n;
    uint32_t npix;
    GuideRec* rec;      // [k * n + i]
    uint8_t* nrec;      // [i]
    float* own;         // [3 i]
};

__device__ __forceinline__ float lum(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

__global__ void __launch_bounds__(kGdThreads) k_gd_generate(CameraGPU cam, Wave w, uint32_t seed,
                                                            float4* __restrict__ rays, PathState* __restrict__ state,
                                                            uint32_t* __restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *count = w.n;  // every path of the wave starts in the queue
    if (i >= w.n) return;
    const uint64_t p = w.p0 + i;
    const uint32_t pixel = (uint32_t)(p % w.npix);
    const uint32_t x = pixel % (uint32_t)cam.width, y = pixel / (uint32_t)cam.width;
    const Philox4x32 r = philox4x32_10((uint32_t)p, (uint32_t)(p >> 32), 0u, 0u, seed, kKeyCamera);
    const float3 d = camera_dir(cam, ((float)x + u01(r.v[0])) / (float)cam.width,
                                ((float)y + u01(r.v[1])) / (float)cam.height);
    rays[2 * i] = make_float4(cam.eye.x, cam.eye.y, cam.eye.z, 1e-4f);
    rays[2 * i + 1] = make_float4(d.x, d.y, d.z, FLT_MAX);
    PathState s;
    s.thr = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(pixel));
    s.id = make_uint4((uint32_t)p, (uint32_t)(p >> 32), 1u, i);
    state[i] = s;
    w.nrec[i] = 0;
    w.own[3 * (size_t)i] = 0.0f;
    w.own[3 * (size_t)i + 1] = 0.0f;
    w.own[3 * (size_t)i + 2] = 0.0f;
}

// warp-aggregated slot in a queue counted by *count
__device__ __forceinline__ uint32_t append_slot(bool take, uint32_t* count)
{
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (m == 0u) return 0;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// counts: [0] next path queue, [1] diffuse queries
__global__ void __launch_bounds__(kGdThreads) k_gd_shade(SceneGPU sc, Wave w, int max_nv, int min_nv, uint32_t seed,
                                                         int rr_mode,
                                                         const float4* __restrict__ rays,
                                                         const PathState* __restrict__ state,
                                                         const lmgpu_hit* __restrict__ hits,
                                                         const uint32_t* __restrict__ d_n,
                                                         float4* __restrict__ out_rays,
                                                         PathState* __restrict__ out_state,
                                                         uint32_t* __restrict__ out_count,
                                                         float* __restrict__ queries,
                                                         PathState* __restrict__ q_state,
                                                         int32_t* __restrict__ q_prim, uint32_t* __restrict__ q_count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *d_n;  // queue length, written by the previous kernels
    bool keep = false, query = false;
    float4 nr0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nr1 = nr0;
    PathState ns;
    float qv[9];
    int32_t qprim = 0;
    if (i < n) {
        const lmgpu_hit h = hits[i];
        const PathState s = state[i];
        const uint32_t path = s.id.w;
        float* acc = w.own + 3 * (size_t)path;
        float c[3] = {0.0f, 0.0f, 0.0f};
        bool emit = false;
        if (h.prim < 0) {
            if (sc.has_env) {
                c[0] = s.thr.x * sc.env_Le[0];
                c[1] = s.thr.y * sc.env_Le[1];
                c[2] = s.thr.z * sc.env_Le[2];
                emit = true;
            }
        }
        float3 gn = f3(0.0f, 0.0f, 0.0f), pos = gn, d = gn;
        int prim = -1;
        if (h.prim >= 0) {
            const float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
            d = f3(r1.x, r1.y, r1.z);
            const float* T = sc.tris + 9 * (size_t)h.prim;
            const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
            gn = normalize3(cross3(p2 - p1, p3 - p1));
            pos = f3(r0.x, r0.y, r0.z) + d * h.t;
            prim = sc.tri_prim[h.prim];
            const PrimGPU& P = sc.prims[prim];
            if (P.is_light && -dot3(d, gn) > 0.0f) {
                c[0] = s.thr.x * P.Le[0];
                c[1] = s.thr.y * P.Le[1];
                c[2] = s.thr.z * P.Le[2];
                emit = true;
            }
        }
        if (emit) {
            if ((int)s.id.z + 1 >= min_nv) {  // min_num_vertices, renderer_pt.cpp:186
                acc[0] += c[0];
                acc[1] += c[1];
                acc[2] += c[2];
            }
            // incident radiance at the path's recorded vertices
            const int nr = w.nrec[path];
            for (int k = 0; k < nr; k++) {
                GuideRec& R = w.rec[(size_t)k * w.n + path];
                R.L.x += c[0] * R.inv_t.x;
                R.L.y += c[1] * R.inv_t.y;
                R.L.z += c[2] * R.inv_t.z;
            }
        }
        if (h.prim >= 0) {
            const PrimGPU& P = sc.prims[prim];
            uint32_t nv = s.id.z;
            const Philox4x32 r = philox4x32_10(s.id.x, s.id.y, nv, 0u, seed, kKeyBounce);
            // roulette: renderer::pt's fixed 0.5, or survival min(1, max(throughput))
            const float survive = rr_mode == 0 ? 0.5f : fminf(1.0f, fmaxf(s.thr.x, fmaxf(s.thr.y, s.thr.z)));
            const float rs = 1.0f / survive;
            if (survive > 0.0f && u01(r.v[3]) <= survive) {
                nv++;
                const bool more = max_nv < 0 || (int)nv < max_nv;
                const float3 wi = d * -1.0f;
                if (more && P.bsdf == LMGPU_BSDF_DIFFUSE && dot3(wi, gn) > 0.0f) {
                    // the guided direction is drawn by k_gd_sample after the network runs
                    query = true;
                    qv[0] = pos.x; qv[1] = pos.y; qv[2] = pos.z;
                    qv[3] = gn.x; qv[4] = gn.y; qv[5] = gn.z;
                    qv[6] = wi.x; qv[7] = wi.y; qv[8] = wi.z;
                    qprim = prim;
                    ns.thr = make_float4(rs * s.thr.x, rs * s.thr.y, rs * s.thr.z, s.thr.w);
                    ns.id = make_uint4(s.id.x, s.id.y, nv, s.id.w);
                } else if (more) {
                    float3 wo;
                    float f[3];
                    if (sample_bsdf(P, gn, wi, u01(r.v[0]), u01(r.v[1]), u01(r.v[2]), wo, f)) {
                        keep = true;
                        nr0 = make_float4(pos.x, pos.y, pos.z, 1e-4f);
                        nr1 = make_float4(wo.x, wo.y, wo.z, FLT_MAX);
                        ns.thr = make_float4(rs * s.thr.x * f[0], rs * s.thr.y * f[1], rs * s.thr.z * f[2],
                                             s.thr.w);
                        ns.id = make_uint4(s.id.x, s.id.y, nv, s.id.w);
                    }
                }
            }
        }
    }
    const uint32_t o = append_slot(keep, out_count);
    if (keep) {
        out_rays[2 * o] = nr0;
        out_rays[2 * o + 1] = nr1;
        out_state[o] = ns;
    }
    const uint32_t qo = append_slot(query, q_count);
    if (query) {
        for (int k = 0; k < 9; k++) queries[9 * (size_t)qo + k] = qv[k];
        q_state[qo] = ns;
        q_prim[qo] = qprim;
    }
}

// Direction sampling at the diffuse vertices from the mixture
// alpha * BSDF + (1 - alpha) * q, and their training records.
__global__ void __launch_bounds__(kGdThreads) k_gd_sample(SceneGPU sc, Wave w, float alpha, uint32_t seed,
                                                          const float* __restrict__ queries,
                                                          const PathState* __restrict__ q_state,
                                                          const int32_t* __restrict__ q_prim,
                                                          const float* __restrict__ raw,
                                                          const uint32_t* __restrict__ d_nq,
                                                          float4* __restrict__ out_rays,
                                                          PathState* __restrict__ out_state,
                                                          uint32_t* __restrict__ out_count)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nq = *d_nq;
    bool keep = false;
    float4 nr0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nr1 = nr0;
    PathState ns;
    if (j < nq) {
        const float* q = queries + 9 * (size_t)j;
        const float3 x = f3(q[0], q[1], q[2]), nrm = f3(q[3], q[4], q[5]);
        const PathState s = q_state[j];
        float z[kOutUsed];
        for (int c = 0; c < kOutUsed; c++) z[c] = raw[(size_t)j * kOutUsed + c];
        Lobes L;
        lobes_from_raw(z, L);
        const Philox4x32 r = philox4x32_10(s.id.x, s.id.y, s.id.z, 2u, seed, kKeyGuide);
        float wdir[3];
        if (u01(r.v[0]) < alpha) {
            float3 b, t;
            basis(nrm, b, t);
            const float3 l = cosine_hemisphere(u01(r.v[1]), u01(r.v[2]));
            const float3 wv = b * l.x + t * l.y + nrm * l.z;
            wdir[0] = wv.x; wdir[1] = wv.y; wdir[2] = wv.z;
        } else {
            mixture_sample(L, u01(r.v[1]), u01(r.v[2]), u01(r.v[3]), wdir);
        }
        const float cosw = nrm.x * wdir[0] + nrm.y * wdir[1] + nrm.z * wdir[2];
        if (cosw > 0.0f) {
            float rr[kLobes];
            const float qpdf = expf(mixture_logpdf(L, wdir, rr));
            const float pdf = alpha * cosw * 0.31830988618379067f + (1.0f - alpha) * qpdf;
            const PrimGPU& P = sc.prims[q_prim[j]];
            const float wgt = cosw * 0.31830988618379067f / pdf;
            float t[3] = {s.thr.x * P.R[0] * wgt, s.thr.y * P.R[1] * wgt, s.thr.z * P.R[2] * wgt};
            if (pdf > 0.0f && (t[0] > 0.0f || t[1] > 0.0f || t[2] > 0.0f)) {
                keep = true;
                nr0 = make_float4(x.x, x.y, x.z, 1e-4f);
                nr1 = make_float4(wdir[0], wdir[1], wdir[2], FLT_MAX);
                ns.thr = make_float4(t[0], t[1], t[2], s.thr.w);
                ns.id = s.id;
                const uint32_t path = s.id.w;
                const int k = w.nrec[path];
                if (k < kMaxRec) {
                    GuideRec& R = w.rec[(size_t)k * w.n + path];
                    R.x = make_float4(x.x, x.y, x.z, pdf);
                    R.n = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
                    R.wo = make_float4(q[6], q[7], q[8], 0.0f);
                    R.wi = make_float4(wdir[0], wdir[1], wdir[2], 0.0f);
                    R.inv_t = make_float4(t[0] > 0.0f ? 1.0f / t[0] : 0.0f, t[1] > 0.0f ? 1.0f / t[1] : 0.0f,
                                          t[2] > 0.0f ? 1.0f / t[2] : 0.0f, 0.0f);
                    R.L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    w.nrec[path] = (uint8_t)(k + 1);
                }
            }
        }
    }
    const uint32_t o = append_slot(keep, out_count);
    if (keep) {
        out_rays[2 * o] = nr0;
        out_rays[2 * o + 1] = nr1;
        out_state[o] = ns;
    }
}

__global__ void k_gd_flush(Wave w, double* __restrict__ film, double* __restrict__ film_sq)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.n) return;
    const uint64_t pix = (w.p0 + i) % w.npix;
    for (int k = 0; k < 3; k++) {
        const float c = w.own[3 * (size_t)i + k];
        if (c != 0.0f) {
            atomicAdd(&film[3 * pix + k], (double)c);
            atomicAdd(&film_sq[3 * pix + k], (double)c * (double)c);
        }
    }
}

// Training samples from the wave's records with L > 0: query, direction,
// weight luminance(L) cos / pdf.  count[0] counts them (capacity cap).
__global__ void k_gd_collect(Wave w, float* __restrict__ tq, float* __restrict__ tdir, float* __restrict__ tw,
                             uint32_t cap, uint32_t* __restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = i < w.n ? w.nrec[i] : 0;
    for (int k = 0; k < kMaxRec; k++) {
        bool take = false;
        GuideRec R;
        float weight = 0.0f;
        if (k < nr) {
            R = w.rec[(size_t)k * w.n + i];
            const float l = lum(R.L.x, R.L.y, R.L.z);
            const float cosw = R.n.x * R.wi.x + R.n.y * R.wi.y + R.n.z * R.wi.z;
            weight = l * cosw / R.x.w;
            take = weight > 0.0f && weight < 1e30f;
        }
        const uint32_t o = append_slot(take, count);
        if (take && o < cap) {
            float* q = tq + 9 * (size_t)o;
            q[0] = R.x.x; q[1] = R.x.y; q[2] = R.x.z;
            q[3] = R.n.x; q[4] = R.n.y; q[5] = R.n.z;
            q[6] = R.wo.x; q[7] = R.wo.y; q[8] = R.wo.z;
            tdir[3 * (size_t)o] = R.wi.x;
            tdir[3 * (size_t)o + 1] = R.wi.y;
            tdir[3 * (size_t)o + 2] = R.wi.z;
            tw[o] = weight;
        }
    }
}

template <typename T>
int grow_buf(T** p, uint64_t* cap, uint64_t count)
{
    if (*cap >= count) return LMGPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    *cap = count;
    return LMGPU_OK;
}

}  // namespace

// Buffers of the guided renderer, kept by the scene between calls.
struct GuidedState {
    GuideRec* rec = nullptr;
    uint64_t rec_cap = 0;
    uint8_t* nrec = nullptr;
    uint64_t nrec_cap = 0;
    float* queries = nullptr;
    uint64_t queries_cap = 0;
    PathState* q_state = nullptr;
    uint64_t q_state_cap = 0;
    int32_t* q_prim = nullptr;
    uint64_t q_prim_cap = 0;
    float* raw = nullptr;
    uint64_t raw_cap = 0;
    float* tq = nullptr;
    uint64_t tq_cap = 0;
    float* tdir = nullptr;
    uint64_t tdir_cap = 0;
    float* tw = nullptr;
    uint64_t tw_cap = 0;
    uint32_t* counts = nullptr;  // [0] next queue, [1] queries, [2] training samples
    uint32_t* h_counts = nullptr;
};

void free_guided(GuidedState* g)
{
    if (!g) return;
    void* ptrs[] = {g->rec, g->nrec, g->queries, g->q_state, g->q_prim, g->raw, g->tq, g->tdir, g->tw, g->counts};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (g->h_counts) cudaFreeHost(g->h_counts);
    delete g;
}

int render_pt_guided(lmgpu_scene* sc, lmgpu_guide* guide, const lmgpu_pt_params* prm,
                     const lmgpu_guiding_params* gp, float* d_image, float* d_variance, cudaStream_t stream,
                     float* last_loss)
{
    const uint64_t npix = (uint64_t)sc->cam.width * sc->cam.height;
    if (npix > kGuidedWave) {
        set_error("lmgpu_render_pt_guided: films above 2^21 pixels are not supported");
        return LMGPU_ERR_INVALID;
    }
    if (!(gp->alpha >= 0.0f && gp->alpha <= 1.0f) || gp->batch == 0) {
        set_error("lmgpu_render_pt_guided: alpha in [0, 1] and batch > 0");
        return LMGPU_ERR_INVALID;
    }
    int rc = clear_film(sc, npix, stream);
    if (rc) return rc;
    if (!sc->guided) sc->guided = new GuidedState();
    GuidedState& G = *sc->guided;
    // a wave: whole passes (one sample per pixel each), up to kGuidedWave paths
    const uint64_t per_wave = kGuidedWave / npix;
    const uint64_t W = npix * (per_wave < prm->spp ? per_wave : prm->spp);
    // the path queues hold a whole wave
    if ((rc = ensure_queues(sc, W))) return rc;
    if ((rc = grow_buf(&G.rec, &G.rec_cap, (uint64_t)kMaxRec * W)) || (rc = grow_buf(&G.nrec, &G.nrec_cap, W)) ||
        (rc = grow_buf(&G.queries, &G.queries_cap, 9 * W)) || (rc = grow_buf(&G.q_state, &G.q_state_cap, W)) ||
        (rc = grow_buf(&G.q_prim, &G.q_prim_cap, W)) || (rc = grow_buf(&G.raw, &G.raw_cap, (uint64_t)kOutUsed * W)))
        return rc;
    const uint64_t tcap = (uint64_t)gp->batch * (gp->max_steps_per_pass > 0 ? gp->max_steps_per_pass : 1);
    if ((rc = grow_buf(&G.tq, &G.tq_cap, 9 * tcap)) || (rc = grow_buf(&G.tdir, &G.tdir_cap, 3 * tcap)) ||
        (rc = grow_buf(&G.tw, &G.tw_cap, tcap)))
        return rc;
    if (!G.counts) {
        if (cudaMalloc(&G.counts, 4 * sizeof(uint32_t)) != cudaSuccess ||
            cudaMallocHost(&G.h_counts, 4 * sizeof(uint32_t)) != cudaSuccess) {
            set_error("lmgpu_render_pt_guided: counter allocation failed");
            return LMGPU_ERR_CUDA;
        }
    }
    const SceneGPU sg = scene_view(sc);
    auto read_counts = [&]() -> int {
        LMGPU_CUDA_TRY(cudaMemcpyAsync(G.h_counts, G.counts, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
        return LMGPU_OK;
    };
    constexpr int kCheckEvery = 8;
    const bool bounded = prm->max_num_vertices >= 0;
    const int maxb = bounded ? (prm->max_num_vertices > 1 ? prm->max_num_vertices - 1 : 0) : (1 << 16);
    float loss = 0.0f;
    const uint64_t total = npix * prm->spp;
    for (uint64_t p0 = 0; p0 < total; p0 += W) {
        Wave w;
        w.p0 = p0;
        w.n = (uint32_t)((total - p0) < W ? (total - p0) : W);
        w.npix = (uint32_t)npix;
        w.rec = G.rec;
        w.nrec = G.nrec;
        w.own = sc->q_own;
        // queue lengths on the device (counts: [0], [1] path queues, [2]
        // network queries, [3] training samples): a wave's bounces are queued
        // without host round trips; with max_num_vertices bounded the queue is
        // empty after max_num_vertices - 1 bounces, otherwise the host checks
        // every kCheckEvery bounces
        const unsigned gblocks = (unsigned)((w.n + kGdThreads - 1) / kGdThreads);
        LMGPU_CUDA_TRY(cudaMemsetAsync(G.counts, 0, 4 * sizeof(uint32_t), stream));
        k_gd_generate<<<gblocks, kGdThreads, 0, stream>>>(sc->cam, w, prm->seed, sc->q_ray[0], sc->q_state[0],
                                                          G.counts);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
        int cur = 0;
        for (int b = 0; b < maxb; b++) {
            if ((rc = launch_trace_dn(sc->accel, sc->q_ray[cur], sc->q_hit, G.counts + cur, w.n, false, stream,
                                      sc->probe)))
                return rc;
            LMGPU_CUDA_TRY(cudaMemsetAsync(G.counts + (1 - cur), 0, sizeof(uint32_t), stream));
            LMGPU_CUDA_TRY(cudaMemsetAsync(G.counts + 2, 0, sizeof(uint32_t), stream));
            k_gd_shade<<<gblocks, kGdThreads, 0, stream>>>(sg, w, prm->max_num_vertices, prm->min_num_vertices,
                                                           prm->seed, (int)gp->rr_mode,
                                                           sc->q_ray[cur], sc->q_state[cur], sc->q_hit, G.counts + cur,
                                                           sc->q_ray[1 - cur], sc->q_state[1 - cur],
                                                           G.counts + (1 - cur), G.queries, G.q_state, G.q_prim,
                                                           G.counts + 2);
            LMGPU_CUDA_TRY(cudaGetLastError());
            if ((rc = guide_forward_device_dn(guide, G.queries, G.counts + 2, w.n, G.raw, stream))) return rc;
            k_gd_sample<<<gblocks, kGdThreads, 0, stream>>>(sg, w, gp->alpha, prm->seed, G.queries, G.q_state,
                                                            G.q_prim, G.raw, G.counts + 2, sc->q_ray[1 - cur],
                                                            sc->q_state[1 - cur], G.counts + (1 - cur));
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 4;
            cur = 1 - cur;
            if (!bounded && (b + 1) % kCheckEvery == 0) {
                if ((rc = read_counts())) return rc;
                if (G.h_counts[cur] == 0) break;
            }
        }
        k_gd_flush<<<(w.n + 255) / 256, 256, 0, stream>>>(w, sc->film, sc->film_sq);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
        if (!gp->train) continue;
        // training samples of this pass, then up to max_steps_per_pass Adam steps
        LMGPU_CUDA_TRY(cudaMemsetAsync(G.counts + 3, 0, sizeof(uint32_t), stream));
        k_gd_collect<<<(w.n + 255) / 256, 256, 0, stream>>>(w, G.tq, G.tdir, G.tw, (uint32_t)tcap,
                                                                       G.counts + 3);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
        if ((rc = read_counts())) return rc;
        const uint64_t nt = G.h_counts[3] < tcap ? G.h_counts[3] : tcap;
        for (uint64_t b0 = 0; b0 < nt; b0 += gp->batch) {
            const uint64_t nb = (nt - b0) < gp->batch ? (nt - b0) : gp->batch;
            if ((rc = guide_gradient_device(guide, G.tq + 9 * b0, G.tdir + 3 * b0, G.tw + b0, nb, stream)) ||
                (rc = guide_adam_device(guide, gp->learning_rate, stream)))
                return rc;
            sc->launches += 3;
            if ((rc = guide_take_loss(guide, stream, &loss))) return rc;
        }
    }
    if (last_loss) *last_loss = loss;
    return finalize_film(sc, prm->spp, d_image, d_variance, stream);
}

}  // namespace lmgpu

using namespace lmgpu;

extern "C" {

int lmgpu_render_pt_guided_device(lmgpu_scene* sc, lmgpu_guide* guide, const lmgpu_pt_params* prm,
                                  const lmgpu_guiding_params* gp, float* d_image, float* d_variance, void* stream,
                                  float* last_loss)
{
    clear_error();
    if (!sc || !guide || !prm || !gp || !d_image) {
        set_error("lmgpu_render_pt_guided: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (prm->spp == 0) {
        set_error("lmgpu_render_pt_guided: spp must be > 0");
        return LMGPU_ERR_INVALID;
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : sc->stream;
    int rc = render_pt_guided(sc, guide, prm, gp, d_image, d_variance, s, last_loss);
    if (rc) return rc;
    uint32_t st = 0;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&st, sc->accel->status, sizeof(st), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & (kStatusBadTree | kStatusStackOverflow)) {
        set_error("lmgpu_render_pt_guided: traversal status " + std::to_string(st));
        return LMGPU_ERR_OVERFLOW;
    }
    return LMGPU_OK;
}

int lmgpu_render_pt_guided(lmgpu_scene* sc, lmgpu_guide* guide, const lmgpu_pt_params* prm,
                           const lmgpu_guiding_params* gp, float* image, float* variance, float* last_loss)
{
    clear_error();
    if (!sc || !image) {
        set_error("lmgpu_render_pt_guided: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    const uint64_t npix = (uint64_t)sc->cam.width * sc->cam.height;
    int rc = ensure_film(sc, npix);
    if (rc) return rc;
    rc = lmgpu_render_pt_guided_device(sc, guide, prm, gp, sc->d_image, variance ? sc->d_variance : nullptr,
                                       sc->stream, last_loss);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(image, sc->d_image, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, sc->stream));
    if (variance)
        LMGPU_CUDA_TRY(cudaMemcpyAsync(variance, sc->d_variance, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost,
                                       sc->stream));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(sc->stream));
    return LMGPU_OK;
}

}  // extern "C"
