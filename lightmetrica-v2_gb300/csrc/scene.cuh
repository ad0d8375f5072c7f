// Device-side scene for the path tracers (the object behind lmgpu_scene*).
#pragma once

#include "accel.cuh"

namespace lmgpu {

// Paths in flight per wave of the wavefront renderers.
constexpr uint64_t kWave = 1ull << 21;

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

    // film: per-pixel sums of splats (FP32) and of their squares (FP64)
    float* film = nullptr;
    double* film_sq = nullptr;
    uint64_t film_cap = 0;
    float* d_image = nullptr;     // staging for the host-pointer render entry points
    float* d_variance = nullptr;

    // two path queues (rays + states), the hits of the current queue, counter
    float4* q_ray[2] = {nullptr, nullptr};
    lmgpu::PathState* q_state[2] = {nullptr, nullptr};
    lmgpu_hit* q_hit = nullptr;
    uint32_t* q_count = nullptr;
    uint32_t* h_count = nullptr;  // pinned host copy
    uint64_t q_cap = 0;
    cudaStream_t stream = nullptr;
};

namespace lmgpu {

int ensure_film(lmgpu_scene* sc, uint64_t npix);
int ensure_queues(lmgpu_scene* sc, uint64_t n);
SceneGPU scene_view(const lmgpu_scene* sc);
int render_pt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream);

}  // namespace lmgpu
