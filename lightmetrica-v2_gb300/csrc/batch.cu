// Batched wavefront path tracing: many scenes and camera views of uneven
// resolution rendered by one wavefront, the estimator of renderer::pt
// (src/liblightmetrica/renderer/renderer_pt.cpp:68-231) for every view.
//
// Structure:
//   * every view is an lmgpu_scene (its triangles, BVH, primitives, camera,
//     optional constant environment); the batch keeps a device table of them;
//   * samples of all views form one index space (view v owns samples
//     [begin_v, begin_v + W_v H_v spp)); a wave of up to `wave` paths may mix
//     views, and every path carries its view;
//   * one bounce = the multi-scene persistent traversal (each ray against its
//     own view's BVH, trace.cu) + k_bt_shade.  Both read the queue length
//     from device memory, so a bounce has a fixed launch shape: it is
//     captured once as a CUDA graph per queue parity and replayed, with no
//     host round trip between bounces;
//   * Russian roulette (probability 0.5) applies once a path has more than
//     rr_depth segments (rr_depth 0: at every hit, as the reference does);
//     either way the estimator is unbiased;
//   * an autotuner (lmgpu_batch_autotune) measures renders of a probe sample
//     count over candidate traversal refill/postpone thresholds and wave
//     sizes, by coordinate descent, and keeps the fastest.
#include "accel.cuh"
#include "bsdf.cuh"
#include "rng.cuh"
#include "scene.cuh"

#include <vector>

namespace lmgpu {
namespace {

constexpr int kBtThreads = 256;
constexpr uint32_t kMaxViews = 255;
constexpr int kBouncesPerSync = 8;
constexpr int kMaxBounces = 1024;

struct BatchView {
    SceneGPU sc;
    CameraGPU cam;
    uint64_t begin;     // first global sample of the view
    uint32_t npix;
    uint32_t pad;
    uint64_t film_off;  // first pixel of the view in the batch film
};

// Per-render arguments the captured bounce graphs read from device memory.
struct RenderArgs {
    uint32_t seed;
    int32_t max_nv;
    int32_t rr_depth;
    uint32_t pad;
};

__device__ __forceinline__ uint32_t find_view(const BatchView* __restrict__ views, uint32_t nviews, uint64_t p)
{
    uint32_t v = 0;
    while (v + 1 < nviews && p >= views[v + 1].begin) v++;
    return v;
}

__global__ void __launch_bounds__(kBtThreads) k_bt_generate(const BatchView* __restrict__ views, uint32_t nviews,
                                                            uint64_t p0, uint32_t n, const RenderArgs* __restrict__ ra,
                                                            float4* __restrict__ rays, PathState* __restrict__ state,
                                                            uint8_t* __restrict__ ray_scene, float* __restrict__ own,
                                                            uint32_t* __restrict__ d_n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *d_n = n;
    if (i >= n) return;
    const uint64_t p = p0 + i;
    const uint32_t v = find_view(views, nviews, p);
    const CameraGPU& cam = views[v].cam;
    const uint32_t pixel = (uint32_t)((p - views[v].begin) % views[v].npix);
    const uint32_t x = pixel % (uint32_t)cam.width, y = pixel / (uint32_t)cam.width;
    const Philox4x32 r = philox4x32_10((uint32_t)p, (uint32_t)(p >> 32), 0u, 0u, ra->seed, kKeyCamera);
    const float rx = ((float)x + u01(r.v[0])) / (float)cam.width;
    const float ry = ((float)y + u01(r.v[1])) / (float)cam.height;
    const float3 d = camera_dir(cam, rx, ry);
    rays[2 * i] = make_float4(cam.eye.x, cam.eye.y, cam.eye.z, 1e-4f);
    rays[2 * i + 1] = make_float4(d.x, d.y, d.z, FLT_MAX);
    PathState s;
    s.thr = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float((v << 24) | pixel));
    s.id = make_uint4((uint32_t)p, (uint32_t)(p >> 32), 1u, i);
    state[i] = s;
    ray_scene[i] = (uint8_t)v;
    own[3 * (size_t)i] = 0.0f;
    own[3 * (size_t)i + 1] = 0.0f;
    own[3 * (size_t)i + 2] = 0.0f;
}

// One bounce for every path in the queue: emission, roulette, BSDF sampling,
// warp-aggregated append to the next queue (grid-stride over *d_n).
__global__ void __launch_bounds__(kBtThreads) k_bt_shade(const BatchView* __restrict__ views,
                                                         const RenderArgs* __restrict__ ra,
                                                         const uint32_t* __restrict__ d_n,
                                                         const float4* __restrict__ rays,
                                                         const PathState* __restrict__ state,
                                                         const lmgpu_hit* __restrict__ hits, float* __restrict__ own,
                                                         float4* __restrict__ out_rays,
                                                         PathState* __restrict__ out_state,
                                                         uint8_t* __restrict__ out_scene,
                                                         uint32_t* __restrict__ d_n_out)
{
    const uint32_t n = *d_n;
    const uint32_t seed = ra->seed;
    const int max_nv = ra->max_nv, rr_depth = ra->rr_depth;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    // every lane of a warp runs the same number of iterations (ballots)
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t round = 0; round < rounds; round++) {
        const uint32_t i = first + round * stride;
        bool keep = false;
        float4 nr0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nr1 = nr0;
        PathState ns;
        uint32_t v = 0;
        if (i < n) {
            const lmgpu_hit h = hits[i];
            const PathState s = state[i];
            const uint32_t tag = __float_as_uint(s.thr.w);
            v = tag >> 24;
            const SceneGPU& sc = views[v].sc;
            float* acc = own + 3 * (size_t)s.id.w;
            if (h.prim < 0) {
                // miss: the view's environment light, if any (scene3.cpp:464-475)
                if (sc.has_env) {
                    acc[0] += s.thr.x * sc.env_Le[0];
                    acc[1] += s.thr.y * sc.env_Le[1];
                    acc[2] += s.thr.z * sc.env_Le[2];
                }
            } else {
                const float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
                const float3 o = f3(r0.x, r0.y, r0.z), d = f3(r1.x, r1.y, r1.z);
                const float* T = sc.tris + 9 * (size_t)h.prim;
                const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
                const float3 gn = normalize3(cross3(p2 - p1, p3 - p1));
                const PrimGPU& P = sc.prims[sc.tri_prim[h.prim]];
                const float3 pos = o + d * h.t;
                uint32_t nv = s.id.z;
                if (P.is_light && -dot3(d, gn) > 0.0f) {
                    acc[0] += s.thr.x * P.Le[0];
                    acc[1] += s.thr.y * P.Le[1];
                    acc[2] += s.thr.z * P.Le[2];
                }
                const Philox4x32 r = philox4x32_10(s.id.x, s.id.y, nv, 0u, seed, kKeyBounce);
                // the path has nv segments now; roulette past rr_depth of them
                const bool rr = (int)nv > rr_depth;
                if (!rr || u01(r.v[3]) <= 0.5f) {
                    const float scale = rr ? 2.0f : 1.0f;
                    nv++;
                    const bool more = max_nv < 0 || (int)nv < max_nv;
                    float3 wo;
                    float f[3];
                    if (more && sample_bsdf(P, gn, d * -1.0f, u01(r.v[0]), u01(r.v[1]), u01(r.v[2]), wo, f)) {
                        keep = true;
                        nr0 = make_float4(pos.x, pos.y, pos.z, 1e-4f);
                        nr1 = make_float4(wo.x, wo.y, wo.z, FLT_MAX);
                        ns.thr = make_float4(scale * s.thr.x * f[0], scale * s.thr.y * f[1], scale * s.thr.z * f[2],
                                             s.thr.w);
                        ns.id = make_uint4(s.id.x, s.id.y, nv, s.id.w);
                    }
                }
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (m == 0u) continue;
        const unsigned lane = threadIdx.x & 31u;
        const unsigned leader = __ffs(m) - 1u;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(d_n_out, (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (keep) {
            const uint32_t o = base + __popc(m & ((1u << lane) - 1u));
            out_rays[2 * o] = nr0;
            out_rays[2 * o + 1] = nr1;
            out_state[o] = ns;
            out_scene[o] = (uint8_t)v;
        }
    }
}

__global__ void k_bt_flush(const BatchView* __restrict__ views, uint32_t nviews, uint64_t p0, uint32_t n,
                           const float* __restrict__ own, double* __restrict__ film, double* __restrict__ film_sq)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t p = p0 + i;
    const uint32_t v = find_view(views, nviews, p);
    const uint64_t pix = views[v].film_off + (p - views[v].begin) % views[v].npix;
    for (int k = 0; k < 3; k++) {
        const float c = own[3 * (size_t)i + k];
        if (c != 0.0f) {
            atomicAdd(&film[3 * pix + k], (double)c);
            atomicAdd(&film_sq[3 * pix + k], (double)c * (double)c);
        }
    }
}

// inv_spp: 1 / spp from the host (FP64 multiplication instead of division).
__global__ void k_bt_finalize(const double* __restrict__ film, const double* __restrict__ film_sq, uint64_t n3,
                              double inv_spp, float* __restrict__ image, float* __restrict__ variance)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const double mean = film[i] * inv_spp;
    image[i] = (float)mean;
    if (variance) {
        const double v = (film_sq[i] - film[i] * mean) * (inv_spp * inv_spp);
        variance[i] = (float)(v > 0.0 ? v : 0.0);
    }
}

template <typename T>
int dev_alloc(T** p, uint64_t count)
{
    if (*p) cudaFree(*p);
    *p = nullptr;
    const cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    return LMGPU_OK;
}

}  // namespace
}  // namespace lmgpu

using namespace lmgpu;

struct lmgpu_batch {
    std::vector<lmgpu_scene*> scenes;  // borrowed
    uint32_t nviews = 0;
    uint64_t total_pix = 0;
    std::vector<uint64_t> film_off;
    AccelView* d_tab = nullptr;
    BatchView* d_views = nullptr;
    std::vector<BatchView> h_views;
    RenderArgs* d_args = nullptr;
    uint32_t* d_status = nullptr;
    double* film = nullptr;
    double* film_sq = nullptr;
    float* d_image = nullptr;  // all views, for the host-pointer entry point
    float* d_variance = nullptr;
    // queues
    uint64_t cap = 0;
    float4* rays[2] = {nullptr, nullptr};
    PathState* state[2] = {nullptr, nullptr};
    uint8_t* ray_scene[2] = {nullptr, nullptr};
    lmgpu_hit* hits = nullptr;
    float* own = nullptr;
    uint32_t* d_n = nullptr;  // [2] queue lengths
    uint32_t* h_n = nullptr;  // pinned
    // tuning and the captured bounce graphs (one per queue parity)
    TraceConfig tune;
    uint64_t wave = 1ull << 21;
    cudaGraphExec_t bounce[2] = {nullptr, nullptr};
    bool graphs_ok = false;
    cudaStream_t stream = nullptr;
    uint64_t launches = 0;
    lmgpu::TraceProbe* probe = nullptr;  // traversal instrumentation (lmgpu_batch_set_trace_profile)
};

namespace lmgpu {
namespace {

void drop_graphs(lmgpu_batch* b)
{
    for (int c = 0; c < 2; c++)
        if (b->bounce[c]) {
            cudaGraphExecDestroy(b->bounce[c]);
            b->bounce[c] = nullptr;
        }
    b->graphs_ok = false;
}

int ensure_batch_queues(lmgpu_batch* b, uint64_t cap)
{
    if (b->cap >= cap) return LMGPU_OK;
    drop_graphs(b);
    int rc;
    for (int c = 0; c < 2; c++)
        if ((rc = dev_alloc(&b->rays[c], 2 * cap)) || (rc = dev_alloc(&b->state[c], cap)) ||
            (rc = dev_alloc(&b->ray_scene[c], cap)))
            return rc;
    if ((rc = dev_alloc(&b->hits, cap)) || (rc = dev_alloc(&b->own, 3 * cap))) return rc;
    b->cap = cap;
    return LMGPU_OK;
}

// Blocks of the shading launch of one bounce.
int shade_grid_of(const lmgpu_batch* b, unsigned* grid)
{
    int dev = 0, sms = 0;
    LMGPU_CUDA_TRY(cudaGetDevice(&dev));
    LMGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const uint64_t by_n = (b->cap + kBtThreads - 1) / kBtThreads;
    *grid = (unsigned)(by_n < (uint64_t)sms * 8 ? by_n : (uint64_t)sms * 8);
    return LMGPU_OK;
}

// One bounce from queue parity c on stream s: traversal of queue c, then
// shading from queue c into queue 1 - c.  probe: NULL inside a capture.
int launch_bounce(lmgpu_batch* b, int c, unsigned shade_grid, cudaStream_t s, TraceProbe* probe)
{
    int rc = launch_trace_multi(b->d_tab, b->nviews, b->rays[c], b->ray_scene[c], b->hits, b->d_n + c, b->cap,
                                false, b->tune, b->d_status, s, probe);
    if (rc) return rc;
    if (cudaMemsetAsync(b->d_n + (1 - c), 0, sizeof(uint32_t), s) != cudaSuccess) return LMGPU_ERR_CUDA;
    k_bt_shade<<<shade_grid, kBtThreads, 0, s>>>(b->d_views, b->d_args, b->d_n + c, b->rays[c], b->state[c], b->hits,
                                                 b->own, b->rays[1 - c], b->state[1 - c], b->ray_scene[1 - c],
                                                 b->d_n + (1 - c));
    return cudaGetLastError() == cudaSuccess ? LMGPU_OK : LMGPU_ERR_CUDA;
}

// Captures one bounce per queue parity c (launch_bounce).
int capture_bounces(lmgpu_batch* b)
{
    if (b->graphs_ok) return LMGPU_OK;
    drop_graphs(b);
    if (trace_grid_cap() <= 0) return LMGPU_ERR_CUDA;  // looked up outside the capture
    unsigned shade_grid = 0;
    int rc = shade_grid_of(b, &shade_grid);
    if (rc) return rc;
    for (int c = 0; c < 2; c++) {
        cudaGraph_t g = nullptr;
        LMGPU_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        rc = launch_bounce(b, c, shade_grid, b->stream, nullptr);
        const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc != LMGPU_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            set_error(std::string("lmgpu_batch: bounce capture failed: ") + cudaGetErrorString(e));
            return LMGPU_ERR_CUDA;
        }
        const cudaError_t ei = cudaGraphInstantiate(&b->bounce[c], g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            set_error(std::string("lmgpu_batch: graph instantiation failed: ") + cudaGetErrorString(ei));
            return LMGPU_ERR_CUDA;
        }
    }
    b->graphs_ok = true;
    return LMGPU_OK;
}

int batch_render(lmgpu_batch* b, const lmgpu_batch_params* prm, float* d_image, float* d_variance, cudaStream_t s)
{
    if (prm->spp == 0 || prm->rr_depth < 0 || prm->rr_depth > kMaxBounces / 2) {
        set_error("lmgpu_batch_render_pt: spp must be > 0 and rr_depth in [0, 512]");
        return LMGPU_ERR_INVALID;
    }
    // sample ranges of the views
    uint64_t begin = 0;
    for (uint32_t v = 0; v < b->nviews; v++) {
        b->h_views[v].begin = begin;
        begin += (uint64_t)b->h_views[v].npix * prm->spp;
    }
    const uint64_t total = begin;
    LMGPU_CUDA_TRY(
        cudaMemcpyAsync(b->d_views, b->h_views.data(), sizeof(BatchView) * b->nviews, cudaMemcpyHostToDevice, s));
    const RenderArgs ra{prm->seed, prm->max_num_vertices, prm->rr_depth, 0u};
    LMGPU_CUDA_TRY(cudaMemcpyAsync(b->d_args, &ra, sizeof(ra), cudaMemcpyHostToDevice, s));
    LMGPU_CUDA_TRY(cudaMemsetAsync(b->d_status, 0, sizeof(uint32_t), s));
    LMGPU_CUDA_TRY(cudaMemsetAsync(b->film, 0, sizeof(double) * 3 * b->total_pix, s));
    LMGPU_CUDA_TRY(cudaMemsetAsync(b->film_sq, 0, sizeof(double) * 3 * b->total_pix, s));
    const uint64_t wave = b->wave < total ? b->wave : total;
    int rc = ensure_batch_queues(b, wave);
    if (rc) return rc;
    // a trace profile launches the bounces one by one (the probe records
    // events and picks the counting traversal per launch); otherwise the
    // captured graphs run
    TraceProbe* probe = b->probe && b->probe->mode != TraceProbe::kOff ? b->probe : nullptr;
    unsigned shade_grid = 0;
    if (probe) {
        if ((rc = shade_grid_of(b, &shade_grid))) return rc;
    } else if ((rc = capture_bounces(b))) {
        return rc;
    }
    // unbounded paths (max_num_vertices -1) stop after kMaxBounces segments;
    // with roulette the survivors are a 2^-(kMaxBounces - rr_depth) fraction
    const int max_bounces = prm->max_num_vertices < 0 ? kMaxBounces : prm->max_num_vertices - 1;
    for (uint64_t p0 = 0; p0 < total; p0 += wave) {
        const uint32_t n = (uint32_t)((total - p0) < wave ? (total - p0) : wave);
        k_bt_generate<<<(n + kBtThreads - 1) / kBtThreads, kBtThreads, 0, s>>>(
            b->d_views, b->nviews, p0, n, b->d_args, b->rays[0], b->state[0], b->ray_scene[0], b->own, b->d_n);
        LMGPU_CUDA_TRY(cudaGetLastError());
        b->launches++;
        int cur = 0;
        for (int k = 0; k < max_bounces; k++) {
            if (probe) {
                if ((rc = launch_bounce(b, cur, shade_grid, s, probe))) return rc;
            } else {
                LMGPU_CUDA_TRY(cudaGraphLaunch(b->bounce[cur], s));
            }
            b->launches += 2;  // traversal + shading
            cur = 1 - cur;
            const bool last = k + 1 == max_bounces;
            if (!last && (k + 1) % kBouncesPerSync == 0) {
                // every few bounces: stop once the queue has emptied
                LMGPU_CUDA_TRY(cudaMemcpyAsync(b->h_n, b->d_n + cur, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
                if (*b->h_n == 0) break;
            }
        }
        k_bt_flush<<<(n + 255) / 256, 256, 0, s>>>(b->d_views, b->nviews, p0, n, b->own, b->film, b->film_sq);
        LMGPU_CUDA_TRY(cudaGetLastError());
        b->launches++;
    }
    const uint64_t n3 = 3 * b->total_pix;
    k_bt_finalize<<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(b->film, b->film_sq, n3, 1.0 / (double)prm->spp,
                                                               d_image, d_variance);
    LMGPU_CUDA_TRY(cudaGetLastError());
    b->launches++;
    uint32_t st = 0;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&st, b->d_status, sizeof(st), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & (kStatusBadTree | kStatusStackOverflow)) {
        set_error("lmgpu_batch_render_pt: traversal status " + std::to_string(st));
        return LMGPU_ERR_OVERFLOW;
    }
    return LMGPU_OK;
}

}  // namespace
}  // namespace lmgpu

extern "C" {

int lmgpu_batch_create(lmgpu_scene* const* scenes, uint32_t nviews, lmgpu_batch** out)
{
    clear_error();
    if (!scenes || !out || nviews == 0 || nviews > kMaxViews) {
        set_error("lmgpu_batch_create: need 1.." + std::to_string(kMaxViews) + " scenes");
        return LMGPU_ERR_INVALID;
    }
    *out = nullptr;
    for (uint32_t v = 0; v < nviews; v++)
        if (!scenes[v]) {
            set_error("lmgpu_batch_create: NULL scene");
            return LMGPU_ERR_INVALID;
        }
    lmgpu_batch* b = new lmgpu_batch();
    auto fail = [&](int rc) {
        lmgpu_batch_destroy(b);
        return rc;
    };
    b->scenes.assign(scenes, scenes + nviews);
    b->nviews = nviews;
    std::vector<AccelView> tab(nviews);
    b->h_views.resize(nviews);
    uint64_t off = 0;
    for (uint32_t v = 0; v < nviews; v++) {
        const lmgpu_scene* sc = scenes[v];
        tab[v].nodes = sc->accel->nodes;
        tab[v].tris = sc->accel->tris;
        tab[v].num_nodes = sc->ntri > 0 ? (uint32_t)sc->accel->num_wide : 0u;
        tab[v].num_tris = (uint32_t)sc->ntri;
        BatchView& bv = b->h_views[v];
        bv.sc = scene_view(sc);
        bv.cam = sc->cam;
        bv.begin = 0;
        bv.npix = (uint32_t)((uint64_t)sc->cam.width * sc->cam.height);
        bv.pad = 0;
        bv.film_off = off;
        if ((uint64_t)sc->cam.width * sc->cam.height >= (1ull << 24)) {
            set_error("lmgpu_batch_create: a view has 2^24 pixels or more");
            return fail(LMGPU_ERR_INVALID);
        }
        b->film_off.push_back(off);
        off += bv.npix;
    }
    b->total_pix = off;
    int rc;
    if ((rc = dev_alloc(&b->d_tab, nviews)) || (rc = dev_alloc(&b->d_views, nviews)) ||
        (rc = dev_alloc(&b->d_args, 1)) || (rc = dev_alloc(&b->d_status, 1)) || (rc = dev_alloc(&b->d_n, 2)) ||
        (rc = dev_alloc(&b->film, 3 * off)) || (rc = dev_alloc(&b->film_sq, 3 * off)) ||
        (rc = dev_alloc(&b->d_image, 3 * off)) || (rc = dev_alloc(&b->d_variance, 3 * off)))
        return fail(rc);
    if (cudaMallocHost((void**)&b->h_n, 2 * sizeof(uint32_t)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMemcpy(b->d_tab, tab.data(), sizeof(AccelView) * nviews, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(b->d_status, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {  // legacy-stream work done before the non-blocking stream runs
        set_error("lmgpu_batch_create: allocation or upload failed");
        return fail(LMGPU_ERR_CUDA);
    }
    *out = b;
    return LMGPU_OK;
}

void lmgpu_batch_destroy(lmgpu_batch* b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    free_probe(b->probe);
    void* ptrs[] = {b->d_tab, b->d_views, b->d_args, b->d_status, b->film, b->film_sq, b->d_image, b->d_variance,
                    b->rays[0], b->rays[1], b->state[0], b->state[1], b->ray_scene[0], b->ray_scene[1], b->hits,
                    b->own, b->d_n};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->h_n) cudaFreeHost(b->h_n);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int lmgpu_batch_set_tuning(lmgpu_batch* b, const lmgpu_batch_tuning* t)
{
    clear_error();
    if (!b || !t || t->refill < 1 || t->refill > 32 || t->postpone < 0 || t->postpone > 32 || t->wave_paths < 1024 ||
        t->wave_paths > (1ull << 26)) {
        set_error("lmgpu_batch_set_tuning: refill 1..32, postpone 0..32, wave_paths 1024..2^26");
        return LMGPU_ERR_INVALID;
    }
    if (b->tune.refill != t->refill || b->tune.postpone != t->postpone) b->graphs_ok = false;
    b->tune.refill = t->refill;
    b->tune.postpone = t->postpone;
    if (t->wave_paths != b->wave) {
        b->wave = t->wave_paths;
        b->graphs_ok = false;
        b->cap = 0;  // queues sized for the new wave
    }
    return LMGPU_OK;
}

int lmgpu_batch_get_tuning(const lmgpu_batch* b, lmgpu_batch_tuning* t)
{
    clear_error();
    if (!b || !t) {
        set_error("lmgpu_batch_get_tuning: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    t->refill = b->tune.refill;
    t->postpone = b->tune.postpone;
    t->wave_paths = b->wave;
    t->probe_ms = 0.0;
    return LMGPU_OK;
}

int lmgpu_batch_render_pt_device(lmgpu_batch* b, const lmgpu_batch_params* prm, float* d_images, float* d_variances,
                                 void* stream)
{
    clear_error();
    if (!b || !prm || !d_images) {
        set_error("lmgpu_batch_render_pt_device: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    return batch_render(b, prm, d_images, d_variances, stream ? (cudaStream_t)stream : b->stream);
}

int lmgpu_batch_render_pt(lmgpu_batch* b, const lmgpu_batch_params* prm, float* const* images,
                          float* const* variances)
{
    clear_error();
    if (!b || !prm || !images) {
        set_error("lmgpu_batch_render_pt: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    for (uint32_t v = 0; v < b->nviews; v++)
        if (!images[v]) {
            set_error("lmgpu_batch_render_pt: NULL image");
            return LMGPU_ERR_INVALID;
        }
    int rc = batch_render(b, prm, b->d_image, variances ? b->d_variance : nullptr, b->stream);
    if (rc) return rc;
    for (uint32_t v = 0; v < b->nviews; v++) {
        const uint64_t o = 3 * b->film_off[v], cnt = 3 * (uint64_t)b->h_views[v].npix;
        LMGPU_CUDA_TRY(cudaMemcpyAsync(images[v], b->d_image + o, sizeof(float) * cnt, cudaMemcpyDeviceToHost,
                                       b->stream));
        if (variances && variances[v])
            LMGPU_CUDA_TRY(cudaMemcpyAsync(variances[v], b->d_variance + o, sizeof(float) * cnt,
                                           cudaMemcpyDeviceToHost, b->stream));
    }
    LMGPU_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return LMGPU_OK;
}

int lmgpu_batch_autotune(lmgpu_batch* b, const lmgpu_batch_params* probe, lmgpu_batch_tuning* out)
{
    clear_error();
    if (!b || !probe) {
        set_error("lmgpu_batch_autotune: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    // coordinate descent over (refill, postpone, wave), each candidate timed
    // as the best of two renders of the probe with CUDA events
    const int refills[] = {2, 4, 8, 16};
    const int postpones[] = {0, 8, 12, 16, 24};
    const uint64_t waves[] = {1ull << 20, 1ull << 21, 1ull << 22, 1ull << 23};
    cudaEvent_t e0, e1;
    LMGPU_CUDA_TRY(cudaEventCreate(&e0));
    LMGPU_CUDA_TRY(cudaEventCreate(&e1));
    auto measure = [&](float& ms) -> int {
        ms = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
            cudaEventRecord(e0, b->stream);
            int rc = batch_render(b, probe, b->d_image, nullptr, b->stream);
            if (rc) return rc;
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float t = 0.0f;
            cudaEventElapsedTime(&t, e0, e1);
            ms = t < ms ? t : ms;
        }
        return LMGPU_OK;
    };
    lmgpu_batch_tuning best{b->tune.refill, b->tune.postpone, b->wave, 0.0};
    float best_ms = 0.0f;
    int rc = measure(best_ms);
    for (int pass = 0; rc == LMGPU_OK && pass < 3; pass++) {
        lmgpu_batch_tuning cand = best;
        if (pass == 0) {
            for (int r : refills) {
                cand.refill = r;
                float ms;
                if ((rc = lmgpu_batch_set_tuning(b, &cand)) || (rc = measure(ms))) break;
                if (ms < best_ms) { best_ms = ms; best = cand; }
            }
        } else if (pass == 1) {
            for (int q : postpones) {
                cand.postpone = q;
                float ms;
                if ((rc = lmgpu_batch_set_tuning(b, &cand)) || (rc = measure(ms))) break;
                if (ms < best_ms) { best_ms = ms; best = cand; }
            }
        } else {
            for (uint64_t w : waves) {
                cand.wave_paths = w;
                float ms;
                if ((rc = lmgpu_batch_set_tuning(b, &cand)) || (rc = measure(ms))) break;
                if (ms < best_ms) { best_ms = ms; best = cand; }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    best.probe_ms = best_ms;
    rc = lmgpu_batch_set_tuning(b, &best);
    if (rc) return rc;
    if (out) *out = best;
    return LMGPU_OK;
}

int lmgpu_batch_launch_count(const lmgpu_batch* b, uint64_t* count)
{
    clear_error();
    if (!b || !count) {
        set_error("lmgpu_batch_launch_count: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    *count = b->launches;
    return LMGPU_OK;
}

int lmgpu_batch_set_trace_profile(lmgpu_batch* b, int mode)
{
    clear_error();
    if (!b) {
        set_error("lmgpu_batch_set_trace_profile: NULL batch");
        return LMGPU_ERR_INVALID;
    }
    return set_probe(&b->probe, mode, "lmgpu_batch_set_trace_profile");
}

int lmgpu_batch_read_trace_profile(lmgpu_batch* b, lmgpu_trace_profile* out)
{
    clear_error();
    if (!b || !out) {
        set_error("lmgpu_batch_read_trace_profile: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    return read_probe(b->probe, out);
}

}  // extern "C"
