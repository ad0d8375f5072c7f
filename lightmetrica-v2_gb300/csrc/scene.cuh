// Device-side scene for the path tracers (the object behind lmgpu_scene*).
#pragma once

#include "accel.cuh"

namespace lmgpu {

// Paths in flight per wave of the wavefront renderers.
constexpr uint64_t kWave = 1ull << 22;

// Philox key words separating the streams a path draws from.
constexpr uint32_t kKeyCamera = 0x43414D45u;  // raster jitter
constexpr uint32_t kKeyBounce = 0x424F554Eu;  // BSDF sample + roulette per bounce

struct PrimGPU {
    int32_t bsdf;
    int32_t is_light;
    float R[3];
    float Le[3];
    float eta1, eta2;
    float ct_eta[3], ct_k[3];
    float roughness;
};

// Pinhole camera: lookat basis (scene3.cpp:213-221) and projection
// parameters (sensor_pinhole.cpp:46-62).
struct CameraGPU {
    float3 eye, vx, vy, vz;
    float tan_fov, aspect;
    int32_t width, height;
};

// Per-path state between bounces (32 bytes): throughput and pixel, then
// path index (64-bit) and number of vertices so far.
struct __align__(16) PathState {
    float4 thr;  // xyz throughput, w = pixel index bits
    uint4 id;    // x, y = path index lo/hi, z = vertices, w = unused
};

// Read-only view passed to kernels by value.
struct SceneGPU {
    const float* tris;
    const int32_t* tri_prim;
    const PrimGPU* prims;
    int32_t has_env;
    float env_Le[3];
};

// Area lights for the bidirectional renderer: the primitives flagged as
// lights, each with its triangles and their area CDF
// (TriangleUtils::CreateTriangleAreaDist, triangleutils.h:40-77).
struct BdptState;
void free_bdpt(BdptState* b);
struct GuidedState;
void free_guided(GuidedState* g);
struct VcmState;
void free_vcm(VcmState* v);

struct LightsGPU {
    int32_t count;
    const int32_t* prims;       // light -> primitive
    const int32_t* prim_light;  // primitive -> light, -1 if not a light
    const int32_t* tri_off;     // light -> first entry in tris; count + 1 entries
    const int32_t* tris;        // global triangle ids grouped by light
    const float* cdf;           // per light (its triangle count + 1) entries, at tri_off[l] + l
    const float* inv_area;      // light -> 1 / total area
};

}  // namespace lmgpu

struct lmgpu_scene {
    lmgpu_accel* accel = nullptr;
    uint64_t ntri = 0;
    float* tris = nullptr;        // float[9] per global triangle id
    int32_t* tri_prim = nullptr;  // primitive index per triangle
    lmgpu::PrimGPU* prims = nullptr;
    uint32_t nprims = 0;
    lmgpu::CameraGPU cam{};
    int32_t has_env = 0;
    float env_Le[3] = {0.0f, 0.0f, 0.0f};
    float sphere_center[3] = {0.0f, 0.0f, 0.0f};  // bounding sphere (scene3.cpp:74-78)
    float sphere_radius = 0.0f;
    lmgpu::LightsGPU lights{};
    void* light_buf = nullptr;  // one allocation behind the pointers of lights

    // film: per-pixel sums of splats and of their squares, in FP64 (splats
    // are FP32 values; FP32 sums drop every splat below half an ulp of the
    // running sum, a visible bias once a pixel holds ~10^4 samples).
    // film / film_sq take the splats of the pixel's own samples (its
    // stratum), film_x / film_x_sq the splats that samples of other pixels
    // make there (light-to-camera connections); the two groups have
    // different distributions, so the variance of the estimate is summed
    // over them separately.
    double* film = nullptr;
    double* film_sq = nullptr;
    double* film_x = nullptr;
    double* film_x_sq = nullptr;
    uint64_t film_cap = 0;
    float* d_image = nullptr;     // staging for the host-pointer render entry points
    float* d_variance = nullptr;

    // two path queues (rays + states), the hits of the current queue, counter
    float4* q_ray[2] = {nullptr, nullptr};
    lmgpu::PathState* q_state[2] = {nullptr, nullptr};
    lmgpu_hit* q_hit = nullptr;
    uint32_t* q_count = nullptr;  // [0], [1] the two path queues' lengths, [2] light-sample queue, [3] spare
    uint32_t* h_count = nullptr;  // pinned host copy
    float* q_own = nullptr;       // [3 path] each path's contributions to its own pixel
    // pending light samples (renderer::ptmis): shadow rays, contributions + pixel, path, hits
    float4* q_nray = nullptr;
    float4* q_nrec = nullptr;
    uint32_t* q_npath = nullptr;
    lmgpu_hit* q_nhit = nullptr;
    uint64_t q_cap = 0;
    cudaStream_t stream = nullptr;
    uint64_t launches = 0;  // kernels launched by the renderers since creation
    lmgpu::BdptState* bdpt = nullptr;
    int bdpt_mis = 0;  // MIS weight of the render in progress (LMGPU_MIS_*)      // buffers of the bidirectional renderer
    lmgpu::GuidedState* guided = nullptr;  // buffers of the guided renderer
    lmgpu::VcmState* vcm = nullptr;        // buffers of the VCM renderer
    lmgpu::TraceProbe* probe = nullptr;    // traversal instrumentation (lmgpu_scene_set_trace_profile)
};

namespace lmgpu {

int ensure_film(lmgpu_scene* sc, uint64_t npix);
// Frees a traversal probe and its events (NULL is ignored).
void free_probe(TraceProbe* p);
// The trace-profile entry points of scenes and batches: set_probe selects the
// mode of *slot (creating or freeing the probe) and clears its record;
// read_probe waits for the device, returns the record and clears it (all
// zero when p is NULL).  fn names the entry point in error messages.
int set_probe(TraceProbe** slot, int mode, const char* fn);
int read_probe(TraceProbe* p, lmgpu_trace_profile* out);
int ensure_queues(lmgpu_scene* sc, uint64_t n);
SceneGPU scene_view(const lmgpu_scene* sc);
int clear_film(lmgpu_scene* sc, uint64_t npix, cudaStream_t stream);
int finalize_film(lmgpu_scene* sc, uint64_t spp, float* d_image, float* d_variance, cudaStream_t stream);
// As finalize_film with spp samples per pixel (not necessarily whole) and
// n_x samples behind the other-samples film.
int finalize_film_nx(lmgpu_scene* sc, double spp, double n_x, float* d_image, float* d_variance,
                     cudaStream_t stream);
// mode: 0 renderer::pt, 1 renderer::ptmis, 2 renderer::ptdirect
int render_pt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream,
              int mode);
int render_bdpt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream);
// renderer::ltdirect (lt.cu)
int render_ltdirect(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance,
                    cudaStream_t stream);

}  // namespace lmgpu
