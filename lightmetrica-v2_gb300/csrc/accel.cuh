// Device-side state of one accel (the object behind lmgpu_accel*).
#pragma once

#include "common.cuh"
#include "../../include/lmgpu.h"

#include <atomic>
#include <mutex>
#include <vector>

namespace lmgpu {
// Tuning knobs of the traversal kernel (see trace.cu): lanes idle before a
// warp refills, and lanes with triangle work below which triangles are
// postponed.
struct TraceConfig {
    int refill = 4;
    int postpone = 12;
};
}  // namespace lmgpu

struct lmgpu_accel {
    int device = 0;
    uint64_t ntri = 0;
    bool built = false;

    // Output of the build: 8-wide compressed nodes and the triangles they
    // reference, both in HBM for the lifetime of the accel.
    lmgpu::WNode* nodes = nullptr;
    lmgpu::WTri* tris = nullptr;
    uint64_t num_wide = 0;
    uint64_t cap_wide = 0;
    uint64_t cap_tris = 0;

    // Global triangle id -> its WTri record (surface geometry at hits).
    int32_t* tri_slot = nullptr;
    // Shading attributes of lmgpu_surface, global triangle order: vertex
    // normals [ntri*9], texcoords [ntri*6], flags [ntri] (bit 0 normals,
    // bit 1 texcoords); attr_ntri = 0 when none are set.
    float* attr_normals = nullptr;
    float* attr_texcoords = nullptr;
    uint8_t* attr_flags = nullptr;
    uint64_t attr_ntri = 0;
    // Surface records read by lmgpu_surface: per global triangle one 128-byte
    // line (positions, vertex normals, texcoords, flags), packed on the device
    // from the triangles and the attributes; surf_ntri = 0 until packed for
    // the current build (read without the lock by queries, so atomic).
    float4* surf = nullptr;
    uint64_t surf_cap = 0;
    std::atomic<uint64_t> surf_ntri{0};

    // Device status word raised by traversal kernels (stack overflow).
    uint32_t* status = nullptr;
    // Traversal counters of the instrumented kernel (4 x u64).
    unsigned long long* counters = nullptr;

    lmgpu_accel_info info{};
    lmgpu::TraceConfig tune;

    // Staging buffers of the host-pointer trace entry point, reused across
    // calls; host_mu serialises callers (Accel3::Intersect may be called from
    // several threads at once, scheduler.cpp:146-183).
    std::mutex host_mu;
    float* stage_rays = nullptr;
    lmgpu_hit* stage_hits = nullptr;
    uint64_t stage_cap = 0;
    cudaStream_t stage_stream[2] = {nullptr, nullptr};
    // Small queries (a single-ray Intersect): rays, hits and a copy of the
    // status word in one pinned, device-mapped host buffer, so a call is one
    // launch, one 4-byte copy and one synchronisation.
    unsigned char* small_host = nullptr;
    unsigned char* small_dev = nullptr;
    // Staging of the host-pointer surface entry point for pageable buffers
    // (rays, hits and planes of one chunk), reused across calls under surf_mu.
    std::mutex surf_mu;
    unsigned char* surf_stage = nullptr;
    uint64_t surf_stage_cap = 0;  // hits per chunk
};

namespace lmgpu {

// Builds the binned-SAH binary tree on the device and collapses it into the
// accel's wide nodes.  d_tris: float[ntri*9] on the device.
// The device address of a page-locked (cudaHostAlloc / cudaHostRegister)
// host buffer, or null for pageable memory and any other kind: the host
// entry points trace such buffers in place across the host link.
inline const void* mapped_host(const void* p)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // an unknown pointer leaves a (non-sticky) error behind
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int build_bvh(lmgpu_accel* a, const float* d_tris, uint64_t ntri, cudaStream_t stream);

struct TraceProbe;

// Launches the traversal kernel over n rays.  probe: see TraceProbe.
int launch_trace(const lmgpu_accel* a, const float4* d_rays, lmgpu_hit* d_hits, uint64_t n, bool anyhit,
                 bool stats, cudaStream_t stream, TraceProbe* probe = nullptr);

// Instrumentation of a renderer's traversal launches (the dominant kernel of
// every wavefront renderer), off unless a scene asks for it.
//   kProbeCount: launches take the counting instantiation, which adds rays,
//                node fetches, triangle fetches and hits into d_counters;
//   kProbeTime:  the production kernel, with a CUDA event pair recorded
//                around each launch (up to kMaxEvents / 2 launches).
// The VCM renderer's photon-merge launches are instrumented the same way
// (counters kMergeCounters.., their own event pairs).
struct TraceProbe {
    static constexpr int kOff = 0, kProbeCount = 1, kProbeTime = 2;
    static constexpr size_t kMaxEvents = 8192;
    static constexpr size_t kMaxMergeEvents = 1024;
    // d_counters: [0, 4) traversal (rays, node fetches, triangle fetches,
    // hits), [4, 8) merges (queries, eye-vertex reads, entries, merges)
    static constexpr int kNumCounters = 8, kMergeCounters = 4;
    int mode = kOff;
    unsigned long long* d_counters = nullptr;  // [kNumCounters], device
    std::vector<cudaEvent_t> events;
    size_t used = 0;           // events recorded since the last read
    uint64_t launches = 0;     // traversal launches since the last read
    bool overflow = false;     // more launches than event pairs
    std::vector<cudaEvent_t> merge_events;
    size_t merge_used = 0;
    uint64_t merge_launches = 0;
};

// As launch_trace with the ray count read from d_n on the device (at most
// max_n), so that launches need no host round trip.  probe: see TraceProbe.
int launch_trace_dn(const lmgpu_accel* a, const float4* d_rays, lmgpu_hit* d_hits, const uint32_t* d_n,
                    uint64_t max_n, bool anyhit, cudaStream_t stream, TraceProbe* probe = nullptr);

// Blocks of the persistent traversal grid (SMs x resident blocks); looked up
// once per process.  Negative on a CUDA error.
int trace_grid_cap();

// One scene's BVH as the multi-scene traversal sees it.
struct AccelView {
    const WNode* nodes;
    const WTri* tris;
    uint32_t num_nodes, num_tris;
};

// Traversal of rays from several scenes in one launch (ray i against
// d_tab[d_ray_scene[i]]), the ray count read from d_n on the device.
// probe: see TraceProbe (NULL inside a graph capture).
int launch_trace_multi(const AccelView* d_tab, uint32_t ntab, const float4* d_rays, const uint8_t* d_ray_scene,
                       lmgpu_hit* d_hits, const uint32_t* d_n, uint64_t max_n, bool anyhit, TraceConfig cfg,
                       uint32_t* d_status, cudaStream_t stream, TraceProbe* probe = nullptr);

}  // namespace lmgpu
