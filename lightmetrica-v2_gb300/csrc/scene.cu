// Scene object of the path tracers and its C ABI (include/lmgpu.h).
#include "scene.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace lmgpu {

namespace {

template <typename T>
int grow(T** p, uint64_t count)
{
    if (*p) cudaFree(*p);
    *p = nullptr;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    return LMGPU_OK;
}

float3 make3(const float* v) { return make_float3(v[0], v[1], v[2]); }
float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
float3 cross(float3 a, float3 b)
{
    return make_float3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
float3 normalize(float3 a)
{
    const float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return make_float3(a.x / l, a.y / l, a.z / l);
}

}  // namespace

void free_probe(TraceProbe* p)
{
    if (!p) return;
    for (cudaEvent_t e : p->events)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : p->merge_events)
        if (e) cudaEventDestroy(e);
    if (p->d_counters) cudaFree(p->d_counters);
    delete p;
}

int set_probe(TraceProbe** slot, int mode, const char* fn)
{
    if (mode < TraceProbe::kOff || mode > TraceProbe::kProbeTime) {
        set_error(std::string(fn) + ": unknown mode");
        return LMGPU_ERR_INVALID;
    }
    if (mode == TraceProbe::kOff) {
        if (*slot) LMGPU_CUDA_TRY(cudaDeviceSynchronize());
        free_probe(*slot);
        *slot = nullptr;
        return LMGPU_OK;
    }
    if (!*slot) {
        *slot = new TraceProbe;
        if (cudaMalloc((void**)&(*slot)->d_counters, TraceProbe::kNumCounters * sizeof(unsigned long long)) !=
            cudaSuccess) {
            free_probe(*slot);
            *slot = nullptr;
            set_error(std::string(fn) + ": counter allocation failed");
            return LMGPU_ERR_CUDA;
        }
    }
    TraceProbe* p = *slot;
    if (mode == TraceProbe::kProbeTime && p->events.empty()) {
        p->events.resize(TraceProbe::kMaxEvents, nullptr);
        for (auto& e : p->events) LMGPU_CUDA_TRY(cudaEventCreate(&e));
        p->merge_events.resize(TraceProbe::kMaxMergeEvents, nullptr);
        for (auto& e : p->merge_events) LMGPU_CUDA_TRY(cudaEventCreate(&e));
    }
    // renders run on non-blocking streams, which the legacy stream's memset
    // does not order: wait for it before any later counting launch
    LMGPU_CUDA_TRY(cudaDeviceSynchronize());
    LMGPU_CUDA_TRY(cudaMemset(p->d_counters, 0, TraceProbe::kNumCounters * sizeof(unsigned long long)));
    LMGPU_CUDA_TRY(cudaDeviceSynchronize());
    p->mode = mode;
    p->used = 0;
    p->launches = 0;
    p->overflow = false;
    p->merge_used = 0;
    p->merge_launches = 0;
    return LMGPU_OK;
}

int read_probe(TraceProbe* p, lmgpu_trace_profile* out)
{
    *out = lmgpu_trace_profile{};
    if (!p) return LMGPU_OK;
    LMGPU_CUDA_TRY(cudaDeviceSynchronize());
    unsigned long long c[TraceProbe::kNumCounters] = {};
    LMGPU_CUDA_TRY(cudaMemcpy(c, p->d_counters, sizeof(c), cudaMemcpyDeviceToHost));
    out->launches = p->launches;
    out->rays = c[0];
    out->node_fetches = c[1];
    out->triangle_fetches = c[2];
    out->hits = c[3];
    const unsigned long long* m = c + TraceProbe::kMergeCounters;
    out->merge_launches = p->merge_launches;
    out->merge_queries = m[0];
    out->merge_eye_vertices = m[1];
    out->merge_entries = m[2];
    out->merges = m[3];
    auto summed = [](const std::vector<cudaEvent_t>& ev, size_t used, double* ms) -> cudaError_t {
        *ms = 0.0;
        for (size_t i = 0; i + 1 < used; i += 2) {
            float e = 0.0f;
            const cudaError_t rc = cudaEventElapsedTime(&e, ev[i], ev[i + 1]);
            if (rc != cudaSuccess) return rc;
            *ms += e;
        }
        return cudaSuccess;
    };
    LMGPU_CUDA_TRY(summed(p->events, p->used, &out->device_ms));
    out->timed_launches = p->used / 2;
    LMGPU_CUDA_TRY(summed(p->merge_events, p->merge_used, &out->merge_ms));
    out->merge_timed_launches = p->merge_used / 2;
    LMGPU_CUDA_TRY(cudaMemset(p->d_counters, 0, sizeof(c)));
    LMGPU_CUDA_TRY(cudaDeviceSynchronize());
    p->used = 0;
    p->launches = 0;
    p->overflow = false;
    p->merge_used = 0;
    p->merge_launches = 0;
    return LMGPU_OK;
}

int ensure_film(lmgpu_scene* sc, uint64_t npix)
{
    if (sc->film_cap >= npix) return LMGPU_OK;
    int rc;
    if ((rc = grow(&sc->film, 3 * npix)) || (rc = grow(&sc->film_sq, 3 * npix)) ||
        (rc = grow(&sc->film_x, 3 * npix)) || (rc = grow(&sc->film_x_sq, 3 * npix)) ||
        (rc = grow(&sc->d_image, 3 * npix)) || (rc = grow(&sc->d_variance, 3 * npix)))
        return rc;
    sc->film_cap = npix;
    return LMGPU_OK;
}

int ensure_queues(lmgpu_scene* sc, uint64_t n)
{
    if (sc->q_cap >= n) return LMGPU_OK;
    int rc;
    for (int i = 0; i < 2; i++)
        if ((rc = grow(&sc->q_ray[i], 2 * n)) || (rc = grow(&sc->q_state[i], n))) return rc;
    if ((rc = grow(&sc->q_hit, n)) || (rc = grow(&sc->q_own, 3 * n)) || (rc = grow(&sc->q_nray, 2 * n)) ||
        (rc = grow(&sc->q_nrec, n)) || (rc = grow(&sc->q_npath, n)) || (rc = grow(&sc->q_nhit, n)))
        return rc;
    sc->q_cap = n;
    return LMGPU_OK;
}

// Mean and variance of the film estimate I = (S_own + S_x) / spp, where
// S_own sums the spp i.i.d. samples of the pixel's stratum and S_x the
// spp * (pixels - 1) i.i.d. samples of the other strata that splat there:
// Var(I) = [spp Var(X_own) + n_x Var(X_x)] / spp^2, each Var(X) estimated as
// sum(x^2) / n - (sum(x) / n)^2.
// The divisors arrive as reciprocals computed once on the host: FP64
// division is a long instruction sequence on this part, FP64 multiplication
// one instruction (and exact for power-of-two sample counts).
__global__ void k_film_finalize(const double* __restrict__ film, const double* __restrict__ film_sq,
                                const double* __restrict__ film_x, const double* __restrict__ film_x_sq, uint32_t n3,
                                double inv_spp, double inv_n_x, float* __restrict__ image, float* __restrict__ variance)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const double so = film[i], sx = film_x[i];
    image[i] = (float)((so + sx) * inv_spp);
    if (variance) {
        double v = film_sq[i] - so * so * inv_spp;
        if (inv_n_x > 0.0) v += film_x_sq[i] - sx * sx * inv_n_x;
        v *= inv_spp * inv_spp;
        variance[i] = (float)(v > 0.0 ? v : 0.0);
    }
}

int clear_film(lmgpu_scene* sc, uint64_t npix, cudaStream_t stream)
{
    int rc = ensure_film(sc, npix);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemsetAsync(sc->film, 0, sizeof(double) * 3 * npix, stream));
    LMGPU_CUDA_TRY(cudaMemsetAsync(sc->film_sq, 0, sizeof(double) * 3 * npix, stream));
    LMGPU_CUDA_TRY(cudaMemsetAsync(sc->film_x, 0, sizeof(double) * 3 * npix, stream));
    LMGPU_CUDA_TRY(cudaMemsetAsync(sc->film_x_sq, 0, sizeof(double) * 3 * npix, stream));
    return LMGPU_OK;
}

int finalize_film_nx(lmgpu_scene* sc, double spp, double n_x, float* d_image, float* d_variance,
                     cudaStream_t stream)
{
    const uint64_t npix = (uint64_t)sc->cam.width * sc->cam.height;
    const uint32_t n3 = (uint32_t)(3 * npix);
    k_film_finalize<<<(n3 + 255) / 256, 256, 0, stream>>>(sc->film, sc->film_sq, sc->film_x, sc->film_x_sq, n3,
                                                         1.0 / spp, n_x > 0.0 ? 1.0 / n_x : 0.0, d_image,
                                                         d_variance);
    LMGPU_CUDA_TRY(cudaGetLastError());
    sc->launches++;
    return LMGPU_OK;
}

int finalize_film(lmgpu_scene* sc, uint64_t spp, float* d_image, float* d_variance, cudaStream_t stream)
{
    // splats from other samples: those of the other pixels' strata
    const uint64_t npix = (uint64_t)sc->cam.width * sc->cam.height;
    return finalize_film_nx(sc, spp, (double)spp * (double)(npix - 1), d_image, d_variance, stream);
}

// Light tables: per light primitive its triangles and their normalised area
// CDF (TriangleUtils::CreateTriangleAreaDist, triangleutils.h:40-77;
// Distribution1D::Normalize, dist.h:55-67) and the inverse total area
// (light_area.cpp:47-60), packed in one device allocation.
int build_lights(lmgpu_scene* sc, const float* tris, const int32_t* tri_prim, uint64_t ntri, const lmgpu_prim* prims,
                 uint32_t nprims)
{
    std::vector<int32_t> prim_light(nprims, -1), light_prims, tri_off(1, 0), ltris;
    std::vector<float> cdf, inv_area;
    for (uint32_t i = 0; i < nprims; i++)
        if (prims[i].is_light) {
            prim_light[i] = (int32_t)light_prims.size();
            light_prims.push_back((int32_t)i);
        }
    std::vector<std::vector<int32_t>> by_light(light_prims.size());
    for (uint64_t k = 0; k < ntri; k++)
        if (prim_light[tri_prim[k]] >= 0) by_light[prim_light[tri_prim[k]]].push_back((int32_t)k);
    for (size_t l = 0; l < light_prims.size(); l++) {
        if (by_light[l].empty()) {
            set_error("lmgpu_scene_create: light primitive " + std::to_string(light_prims[l]) + " has no triangles");
            return LMGPU_ERR_INVALID;
        }
        const size_t c0 = cdf.size();
        cdf.push_back(0.0f);
        float sum = 0.0f;
        for (int32_t k : by_light[l]) {
            const float* T = tris + 9 * (size_t)k;
            const float3 c = cross(sub3(make3(T + 3), make3(T)), sub3(make3(T + 6), make3(T)));
            const float area = std::sqrt(c.x * c.x + c.y * c.y + c.z * c.z) * 0.5f;
            cdf.push_back(cdf.back() + area);
            sum += area;
            ltris.push_back(k);
        }
        const float total = cdf.back();
        for (size_t q = c0; q < cdf.size(); q++) cdf[q] /= total;
        inv_area.push_back(1.0f / sum);
        tri_off.push_back((int32_t)ltris.size());
    }
    const size_t nl = light_prims.size();
    const size_t bytes = 4 * (nl + nprims + tri_off.size() + ltris.size() + cdf.size() + inv_area.size()) + 4;
    std::vector<unsigned char> host(bytes);
    size_t off = 0;
    auto put = [&](const void* src, size_t n) {
        const size_t at = off;
        if (n) std::memcpy(host.data() + off, src, n);
        off += n;
        return at;
    };
    const size_t o_prims = put(light_prims.data(), 4 * nl), o_pl = put(prim_light.data(), 4 * (size_t)nprims),
                 o_off = put(tri_off.data(), 4 * tri_off.size()), o_tris = put(ltris.data(), 4 * ltris.size()),
                 o_cdf = put(cdf.data(), 4 * cdf.size()), o_ia = put(inv_area.data(), 4 * inv_area.size());
    if (cudaMalloc(&sc->light_buf, bytes) != cudaSuccess ||
        cudaMemcpy(sc->light_buf, host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {  // renders read it on non-blocking streams
        set_error("lmgpu_scene_create: light table upload failed");
        return LMGPU_ERR_CUDA;
    }
    unsigned char* b = (unsigned char*)sc->light_buf;
    LightsGPU& L = sc->lights;
    L.count = (int32_t)nl;
    L.prims = (const int32_t*)(b + o_prims);
    L.prim_light = (const int32_t*)(b + o_pl);
    L.tri_off = (const int32_t*)(b + o_off);
    L.tris = (const int32_t*)(b + o_tris);
    L.cdf = (const float*)(b + o_cdf);
    L.inv_area = (const float*)(b + o_ia);
    return LMGPU_OK;
}

SceneGPU scene_view(const lmgpu_scene* sc)
{
    SceneGPU g;
    g.tris = sc->tris;
    g.tri_prim = sc->tri_prim;
    g.prims = sc->prims;
    g.has_env = sc->has_env;
    for (int k = 0; k < 3; k++) g.env_Le[k] = sc->env_Le[k];
    return g;
}

}  // namespace lmgpu

using namespace lmgpu;

extern "C" {

int lmgpu_scene_create(const float* tris, const int32_t* tri_prim, uint64_t ntri, const lmgpu_prim* prims,
                       uint32_t nprims, const lmgpu_camera* cam, lmgpu_scene** out)
{
    clear_error();
    if (!out || !cam || (ntri > 0 && (!tris || !tri_prim)) || (nprims > 0 && !prims)) {
        set_error("lmgpu_scene_create: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    *out = nullptr;
    if (cam->width <= 0 || cam->height <= 0 || !(cam->fov_deg > 0.0f && cam->fov_deg < 180.0f)) {
        set_error("lmgpu_scene_create: bad camera (width, height > 0, 0 < fov < 180)");
        return LMGPU_ERR_INVALID;
    }
    for (uint64_t i = 0; i < ntri; i++) {
        if (tri_prim[i] < 0 || (uint32_t)tri_prim[i] >= nprims) {
            set_error("lmgpu_scene_create: triangle " + std::to_string(i) + " names primitive " +
                      std::to_string(tri_prim[i]) + " of " + std::to_string(nprims));
            return LMGPU_ERR_INVALID;
        }
    }
    for (uint32_t i = 0; i < nprims; i++) {
        if (prims[i].bsdf < LMGPU_BSDF_NULL || prims[i].bsdf > LMGPU_BSDF_COOK_TORRANCE) {
            set_error("lmgpu_scene_create: unsupported bsdf kind " + std::to_string(prims[i].bsdf));
            return LMGPU_ERR_INVALID;
        }
    }
    lmgpu_scene* sc = new lmgpu_scene();
    auto fail = [&](int rc) {
        lmgpu_scene_destroy(sc);
        return rc;
    };
    int rc = lmgpu_accel_create(&sc->accel);
    if (rc) return fail(rc);
    if (cudaStreamCreateWithFlags(&sc->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost((void**)&sc->h_count, 4 * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc((void**)&sc->q_count, 4 * sizeof(uint32_t)) != cudaSuccess) {
        set_error("lmgpu_scene_create: stream or buffer allocation failed");
        return fail(LMGPU_ERR_CUDA);
    }
    sc->ntri = ntri;
    sc->nprims = nprims;
    if ((rc = grow(&sc->tris, 9 * ntri)) || (rc = grow(&sc->tri_prim, ntri)) || (rc = grow(&sc->prims, nprims)))
        return fail(rc);
    static_assert(sizeof(PrimGPU) == sizeof(lmgpu_prim), "primitive layout");
    if (cudaMemcpy(sc->tris, tris, sizeof(float) * 9 * ntri, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(sc->tri_prim, tri_prim, sizeof(int32_t) * ntri, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(sc->prims, prims, sizeof(PrimGPU) * nprims, cudaMemcpyHostToDevice) != cudaSuccess ||
        // a copy from pageable memory may return before its DMA ends, and the
        // build runs on the scene's non-blocking stream: wait for the copies
        cudaDeviceSynchronize() != cudaSuccess) {
        set_error("lmgpu_scene_create: upload failed");
        return fail(LMGPU_ERR_CUDA);
    }
    rc = build_bvh(sc->accel, sc->tris, ntri, sc->stream);
    if (rc) return fail(rc);
    rc = build_lights(sc, tris, tri_prim, ntri, prims, nprims);
    if (rc) return fail(rc);
    // lookat basis (scene3.cpp:213-221) and pinhole parameters (sensor_pinhole.cpp:46-62)
    const float3 eye = make3(cam->eye), center = make3(cam->center), up = make3(cam->up);
    CameraGPU& c = sc->cam;
    c.eye = eye;
    c.vz = normalize(sub3(eye, center));
    c.vx = normalize(cross(up, c.vz));
    c.vy = cross(c.vz, c.vx);
    c.tan_fov = std::tan(cam->fov_deg * 3.14159265358979323846f / 180.0f * 0.5f);
    c.aspect = (float)cam->width / (float)cam->height;
    c.width = cam->width;
    c.height = cam->height;
    // bounding sphere of the mesh vertices and the sensor position
    // (scene3.cpp:52-78, sensor_pinhole.cpp:158-161), radius grown by 1%
    float lo[3] = {eye.x, eye.y, eye.z}, hi[3] = {eye.x, eye.y, eye.z};
    for (uint64_t i = 0; i < 3 * ntri; i++)
        for (int k = 0; k < 3; k++) {
            lo[k] = std::fmin(lo[k], tris[3 * i + k]);
            hi[k] = std::fmax(hi[k], tris[3 * i + k]);
        }
    float r2 = 0.0f;
    for (int k = 0; k < 3; k++) {
        sc->sphere_center[k] = (hi[k] + lo[k]) * 0.5f;
        r2 += (sc->sphere_center[k] - hi[k]) * (sc->sphere_center[k] - hi[k]);
    }
    sc->sphere_radius = std::sqrt(r2) * 1.01f;
    *out = sc;
    return LMGPU_OK;
}

int lmgpu_scene_set_environment(lmgpu_scene* sc, const float* Le)
{
    clear_error();
    if (!sc) {
        set_error("lmgpu_scene_set_environment: NULL scene");
        return LMGPU_ERR_INVALID;
    }
    sc->has_env = Le ? 1 : 0;
    for (int k = 0; k < 3; k++) sc->env_Le[k] = Le ? Le[k] : 0.0f;
    return LMGPU_OK;
}

void lmgpu_scene_destroy(lmgpu_scene* sc)
{
    if (!sc) return;
    if (sc->stream) cudaStreamSynchronize(sc->stream);
    lmgpu_accel_destroy(sc->accel);
    free_bdpt(sc->bdpt);
    free_guided(sc->guided);
    free_vcm(sc->vcm);
    void* ptrs[] = {sc->tris, sc->tri_prim, sc->prims, sc->film, sc->film_sq, sc->film_x, sc->film_x_sq,
                    sc->d_image, sc->d_variance,
                    sc->q_ray[0], sc->q_ray[1], sc->q_state[0], sc->q_state[1], sc->q_hit, sc->q_count,
                    sc->q_own, sc->q_nray, sc->q_nrec, sc->q_npath, sc->q_nhit,
                    sc->light_buf};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (sc->h_count) cudaFreeHost(sc->h_count);
    if (sc->stream) cudaStreamDestroy(sc->stream);
    free_probe(sc->probe);
    delete sc;
}

int lmgpu_scene_launch_count(const lmgpu_scene* sc, uint64_t* count)
{
    clear_error();
    if (!sc || !count) {
        set_error("lmgpu_scene_launch_count: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    *count = sc->launches;
    return LMGPU_OK;
}

int lmgpu_scene_set_trace_profile(lmgpu_scene* sc, int mode)
{
    clear_error();
    if (!sc) {
        set_error("lmgpu_scene_set_trace_profile: NULL scene");
        return LMGPU_ERR_INVALID;
    }
    return set_probe(&sc->probe, mode, "lmgpu_scene_set_trace_profile");
}

int lmgpu_scene_read_trace_profile(lmgpu_scene* sc, lmgpu_trace_profile* out)
{
    clear_error();
    if (!sc || !out) {
        set_error("lmgpu_scene_read_trace_profile: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    return read_probe(sc->probe, out);
}

int lmgpu_scene_accel(const lmgpu_scene* sc, const lmgpu_accel** accel)
{
    clear_error();
    if (!sc || !accel) {
        set_error("lmgpu_scene_accel: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    *accel = sc->accel;
    return LMGPU_OK;
}

}  // extern "C"

namespace {

using RenderFn = int (*)(lmgpu_scene*, const lmgpu_pt_params*, float*, float*, cudaStream_t);

int render_pt_plain(lmgpu_scene* sc, const lmgpu_pt_params* p, float* img, float* var, cudaStream_t s)
{
    return render_pt(sc, p, img, var, s, 0);
}

int render_pt_nee(lmgpu_scene* sc, const lmgpu_pt_params* p, float* img, float* var, cudaStream_t s)
{
    return render_pt(sc, p, img, var, s, 1);
}

int render_pt_direct(lmgpu_scene* sc, const lmgpu_pt_params* p, float* img, float* var, cudaStream_t s)
{
    return render_pt(sc, p, img, var, s, 2);
}

int render_device(const char* name, RenderFn fn, lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image,
                  float* d_variance, void* stream)
{
    if (!sc || !prm || !d_image) {
        set_error(std::string(name) + ": NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (prm->spp == 0 || (uint64_t)sc->cam.width * sc->cam.height * prm->spp > (1ull << 40)) {
        set_error(std::string(name) + ": spp must be in [1, 2^40 / pixels]");
        return LMGPU_ERR_INVALID;
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : sc->stream;
    int rc = fn(sc, prm, d_image, d_variance, s);
    if (rc) return rc;
    uint32_t st = 0;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&st, sc->accel->status, sizeof(st), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & (kStatusBadTree | kStatusStackOverflow)) {
        set_error(std::string(name) + ": traversal status " + std::to_string(st));
        return LMGPU_ERR_OVERFLOW;
    }
    return LMGPU_OK;
}

int render_host(const char* name, RenderFn fn, lmgpu_scene* sc, const lmgpu_pt_params* prm, float* image,
                float* variance)
{
    if (!sc || !prm || !image) {
        set_error(std::string(name) + ": NULL argument");
        return LMGPU_ERR_INVALID;
    }
    const uint64_t npix = (uint64_t)sc->cam.width * sc->cam.height;
    int rc = ensure_film(sc, npix);
    if (rc) return rc;
    rc = render_device(name, fn, sc, prm, sc->d_image, variance ? sc->d_variance : nullptr, sc->stream);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(image, sc->d_image, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, sc->stream));
    if (variance)
        LMGPU_CUDA_TRY(cudaMemcpyAsync(variance, sc->d_variance, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost,
                                       sc->stream));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(sc->stream));
    return LMGPU_OK;
}

}  // namespace

extern "C" {

int lmgpu_render_pt_device(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance,
                           void* stream)
{
    clear_error();
    return render_device("lmgpu_render_pt_device", render_pt_plain, sc, prm, d_image, d_variance, stream);
}

int lmgpu_render_pt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* image, float* variance)
{
    clear_error();
    return render_host("lmgpu_render_pt", render_pt_plain, sc, prm, image, variance);
}

int lmgpu_render_ptmis_device(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance,
                              void* stream)
{
    clear_error();
    return render_device("lmgpu_render_ptmis_device", render_pt_nee, sc, prm, d_image, d_variance, stream);
}

int lmgpu_render_ptmis(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* image, float* variance)
{
    clear_error();
    return render_host("lmgpu_render_ptmis", render_pt_nee, sc, prm, image, variance);
}

int lmgpu_render_ptdirect_device(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance,
                                 void* stream)
{
    clear_error();
    return render_device("lmgpu_render_ptdirect_device", render_pt_direct, sc, prm, d_image, d_variance, stream);
}

int lmgpu_render_ptdirect(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* image, float* variance)
{
    clear_error();
    return render_host("lmgpu_render_ptdirect", render_pt_direct, sc, prm, image, variance);
}

int lmgpu_render_ltdirect_device(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance,
                                 void* stream)
{
    clear_error();
    return render_device("lmgpu_render_ltdirect_device", render_ltdirect, sc, prm, d_image, d_variance, stream);
}

int lmgpu_render_ltdirect(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* image, float* variance)
{
    clear_error();
    return render_host("lmgpu_render_ltdirect", render_ltdirect, sc, prm, image, variance);
}

int lmgpu_render_bdpt_device(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance,
                             void* stream)
{
    clear_error();
    return render_device("lmgpu_render_bdpt_device", render_bdpt, sc, prm, d_image, d_variance, stream);
}

int lmgpu_render_bdpt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* image, float* variance)
{
    clear_error();
    return render_host("lmgpu_render_bdpt", render_bdpt, sc, prm, image, variance);
}

int lmgpu_render_bdpt_mis(lmgpu_scene* sc, const lmgpu_pt_params* prm, int mis, float* image, float* variance)
{
    clear_error();
    if (!sc || (mis != LMGPU_MIS_POWER && mis != LMGPU_MIS_SIMPLE)) {
        set_error("lmgpu_render_bdpt_mis: NULL scene or unknown MIS weight");
        return LMGPU_ERR_INVALID;
    }
    sc->bdpt_mis = mis;
    const int rc = render_host("lmgpu_render_bdpt_mis", render_bdpt, sc, prm, image, variance);
    sc->bdpt_mis = LMGPU_MIS_POWER;
    return rc;
}

int lmgpu_render_bdpt_mis_device(lmgpu_scene* sc, const lmgpu_pt_params* prm, int mis, float* d_image,
                                 float* d_variance, void* stream)
{
    clear_error();
    if (!sc || (mis != LMGPU_MIS_POWER && mis != LMGPU_MIS_SIMPLE)) {
        set_error("lmgpu_render_bdpt_mis_device: NULL scene or unknown MIS weight");
        return LMGPU_ERR_INVALID;
    }
    sc->bdpt_mis = mis;
    const int rc = render_device("lmgpu_render_bdpt_mis_device", render_bdpt, sc, prm, d_image, d_variance, stream);
    sc->bdpt_mis = LMGPU_MIS_POWER;
    return rc;
}

}  // extern "C"
