// C ABI of the lmgpu library (declared in include/lmgpu.h).
#include "accel.cuh"

#include <cstring>
#include <string>

namespace lmgpu {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

}  // namespace lmgpu

using namespace lmgpu;

namespace {

int check_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error(std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count is 0"));
        return LMGPU_ERR_NO_DEVICE;
    }
    return LMGPU_OK;
}

// The traversal status word as an error code and message.
int status_error(uint32_t st)
{
    if (st & kStatusBadTree) {
        set_error("traversal met an out-of-range node or triangle index (malformed BVH)");
        return LMGPU_ERR_OVERFLOW;
    }
    if (st & kStatusStackOverflow) {
        set_error("traversal stack bound exceeded (results of some rays are incomplete)");
        return LMGPU_ERR_OVERFLOW;
    }
    return LMGPU_OK;
}

int read_status(const lmgpu_accel* a, cudaStream_t stream)
{
    uint32_t st = 0;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&st, a->status, sizeof(st), cudaMemcpyDeviceToHost, stream));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
    return status_error(st);
}

// Rays staged through device memory at once by the host-buffer entry point
// (rays 32 B + hits 16 B per ray: 384 MiB for the two halves).
constexpr uint64_t kHostBatch = 8ull << 20;

// Queries of at most kSmallRays rays take the mapped-buffer path.
constexpr uint64_t kSmallRays = 256;
constexpr size_t kSmallHitsOff = kSmallRays * 32;
constexpr size_t kSmallStatusOff = kSmallHitsOff + kSmallRays * sizeof(lmgpu_hit);
constexpr size_t kSmallBytes = kSmallStatusOff + 16;

// n <= kSmallRays rays from host memory: the kernel reads the rays from and
// writes the hits to the pinned, mapped buffer directly.  Caller holds host_mu.
int trace_small(lmgpu_accel* a, const float* rays, lmgpu_hit* hits, uint64_t n, int anyhit)
{
    if (!a->small_host) {
        void* h = nullptr;
        void* d = nullptr;
        LMGPU_CUDA_TRY(cudaHostAlloc(&h, kSmallBytes, cudaHostAllocMapped));
        if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) {
            cudaFreeHost(h);
            set_error("lmgpu_trace: mapped staging buffer unavailable");
            return LMGPU_ERR_CUDA;
        }
        a->small_host = static_cast<unsigned char*>(h);
        a->small_dev = static_cast<unsigned char*>(d);
    }
    if (!a->stage_stream[0]) LMGPU_CUDA_TRY(cudaStreamCreateWithFlags(&a->stage_stream[0], cudaStreamNonBlocking));
    cudaStream_t s = a->stage_stream[0];
    std::memcpy(a->small_host, rays, n * 32);
    int rc = launch_trace(a, reinterpret_cast<const float4*>(a->small_dev),
                          reinterpret_cast<lmgpu_hit*>(a->small_dev + kSmallHitsOff), n, anyhit != 0, false, s);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(a->small_host + kSmallStatusOff, a->status, sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(hits, a->small_host + kSmallHitsOff, n * sizeof(lmgpu_hit));
    uint32_t st = 0;
    std::memcpy(&st, a->small_host + kSmallStatusOff, sizeof(st));
    return status_error(st);
}

}  // namespace

extern "C" {

const char* lmgpu_version(void) { return "lmgpu 0.1 (sm_103a)"; }

const char* lmgpu_last_error(void) { return g_last_error.c_str(); }

int lmgpu_accel_create(lmgpu_accel** out)
{
    clear_error();
    if (!out) {
        set_error("lmgpu_accel_create: out is NULL");
        return LMGPU_ERR_INVALID;
    }
    *out = nullptr;
    int rc = check_device();
    if (rc) return rc;
    lmgpu_accel* a = new lmgpu_accel();
    cudaGetDevice(&a->device);
    if (cudaMalloc((void**)&a->status, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc((void**)&a->counters, 4 * sizeof(unsigned long long)) != cudaSuccess) {
        set_error("lmgpu_accel_create: cudaMalloc failed");
        if (a->status) cudaFree(a->status);
        delete a;
        return LMGPU_ERR_CUDA;
    }
    // the legacy stream's memset is not ordered with the library's
    // non-blocking streams: finish it before the accel is used
    if (cudaMemset(a->status, 0, sizeof(uint32_t)) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        set_error("lmgpu_accel_create: status initialisation failed");
        lmgpu_accel_destroy(a);
        return LMGPU_ERR_CUDA;
    }
    *out = a;
    return LMGPU_OK;
}

void lmgpu_accel_destroy(lmgpu_accel* a)
{
    if (!a) return;
    if (a->nodes) cudaFree(a->nodes);
    if (a->tris) cudaFree(a->tris);
    if (a->tri_slot) cudaFree(a->tri_slot);
    if (a->attr_normals) cudaFree(a->attr_normals);
    if (a->attr_texcoords) cudaFree(a->attr_texcoords);
    if (a->attr_flags) cudaFree(a->attr_flags);
    if (a->surf) cudaFree(a->surf);
    if (a->status) cudaFree(a->status);
    if (a->counters) cudaFree(a->counters);
    if (a->stage_rays) cudaFree(a->stage_rays);
    if (a->stage_hits) cudaFree(a->stage_hits);
    for (int i = 0; i < 2; i++)
        if (a->stage_stream[i]) cudaStreamDestroy(a->stage_stream[i]);
    if (a->small_host) cudaFreeHost(a->small_host);
    if (a->surf_stage) cudaFree(a->surf_stage);
    delete a;
}

int lmgpu_accel_build_device(lmgpu_accel* a, const float* d_tris, uint64_t ntri, void* stream)
{
    clear_error();
    if (!a || (ntri > 0 && !d_tris)) {
        set_error("lmgpu_accel_build_device: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    return build_bvh(a, d_tris, ntri, (cudaStream_t)stream);
}

int lmgpu_accel_build(lmgpu_accel* a, const float* tris, uint64_t ntri)
{
    clear_error();
    if (!a || (ntri > 0 && !tris)) {
        set_error("lmgpu_accel_build: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (ntri == 0) return build_bvh(a, nullptr, 0, 0);
    float* d = nullptr;
    LMGPU_CUDA_TRY(cudaMalloc((void**)&d, sizeof(float) * 9 * ntri));
    cudaError_t e = cudaMemcpy(d, tris, sizeof(float) * 9 * ntri, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        set_error(std::string("lmgpu_accel_build: copy: ") + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    int rc = build_bvh(a, d, ntri, 0);
    cudaFree(d);
    return rc;
}

int lmgpu_accel_get_info(const lmgpu_accel* a, lmgpu_accel_info* info)
{
    clear_error();
    if (!a || !info) {
        set_error("lmgpu_accel_get_info: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (!a->built) {
        set_error("lmgpu_accel_get_info: accel not built");
        return LMGPU_ERR_NOT_BUILT;
    }
    *info = a->info;
    return LMGPU_OK;
}

int lmgpu_trace_device(const lmgpu_accel* a, const float* d_rays, lmgpu_hit* d_hits, uint64_t n, int anyhit,
                       void* stream)
{
    clear_error();
    if (!a || (n > 0 && (!d_rays || !d_hits))) {
        set_error("lmgpu_trace_device: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (!a->built) {
        set_error("lmgpu_trace_device: accel not built");
        return LMGPU_ERR_NOT_BUILT;
    }
    if (((uintptr_t)d_rays & 15u) || ((uintptr_t)d_hits & 15u)) {
        set_error("lmgpu_trace_device: rays and hits must be 16-byte aligned");
        return LMGPU_ERR_INVALID;
    }
    return launch_trace(a, reinterpret_cast<const float4*>(d_rays), d_hits, n, anyhit != 0, false,
                        (cudaStream_t)stream);
}

int lmgpu_trace_stats_device(const lmgpu_accel* a, const float* d_rays, lmgpu_hit* d_hits, uint64_t n, int anyhit,
                             void* stream, lmgpu_trace_stats* stats)
{
    clear_error();
    if (!a || !stats || (n > 0 && (!d_rays || !d_hits))) {
        set_error("lmgpu_trace_stats_device: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (!a->built) {
        set_error("lmgpu_trace_stats_device: accel not built");
        return LMGPU_ERR_NOT_BUILT;
    }
    if (((uintptr_t)d_rays & 15u) || ((uintptr_t)d_hits & 15u)) {
        set_error("lmgpu_trace_stats_device: rays and hits must be 16-byte aligned");
        return LMGPU_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    LMGPU_CUDA_TRY(cudaMemsetAsync(a->counters, 0, 4 * sizeof(unsigned long long), s));
    int rc = launch_trace(a, reinterpret_cast<const float4*>(d_rays), d_hits, n, anyhit != 0, true, s);
    if (rc) return rc;
    unsigned long long c[4];
    LMGPU_CUDA_TRY(cudaMemcpyAsync(c, a->counters, sizeof(c), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    stats->rays = c[0];
    stats->node_fetches = c[1];
    stats->triangle_fetches = c[2];
    stats->hits = c[3];
    return read_status(a, s);
}

int lmgpu_trace(const lmgpu_accel* ca, const float* rays, lmgpu_hit* hits, uint64_t n, int anyhit)
{
    clear_error();
    if (!ca || (n > 0 && (!rays || !hits))) {
        set_error("lmgpu_trace: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (!ca->built) {
        set_error("lmgpu_trace: accel not built");
        return LMGPU_ERR_NOT_BUILT;
    }
    if (n == 0) return LMGPU_OK;
    // The staging buffers are state of the accel object, not of the query.
    lmgpu_accel* a = const_cast<lmgpu_accel*>(ca);
    std::lock_guard<std::mutex> lock(a->host_mu);
    if (n <= kSmallRays) return trace_small(a, rays, hits, n, anyhit);
    // Page-locked host buffers are mapped into the device's address space:
    // the kernel reads the rays and writes the hits across the host link
    // itself, with no staging copies and one launch.
    const void* d_rays = mapped_host(rays);
    void* d_hits = const_cast<void*>(mapped_host(hits));
    if (d_rays && d_hits && !(((uintptr_t)d_rays | (uintptr_t)d_hits) & 15u)) {
        if (!a->stage_stream[0])
            LMGPU_CUDA_TRY(cudaStreamCreateWithFlags(&a->stage_stream[0], cudaStreamNonBlocking));
        const int rc = launch_trace(a, static_cast<const float4*>(d_rays), static_cast<lmgpu_hit*>(d_hits), n,
                                    anyhit != 0, false, a->stage_stream[0]);
        if (rc) return rc;
        return read_status(a, a->stage_stream[0]);
    }
    // Two staging halves; batch i is copied in on stream i%2 while the other
    // stream traces or copies out, so host<->device copies overlap traversal.
    const uint64_t half = kHostBatch / 2;
    const uint64_t want = n < half ? n : half;
    if (a->stage_cap < want) {
        if (a->stage_rays) cudaFree(a->stage_rays);
        if (a->stage_hits) cudaFree(a->stage_hits);
        a->stage_rays = nullptr;
        a->stage_hits = nullptr;
        a->stage_cap = 0;
        LMGPU_CUDA_TRY(cudaMalloc((void**)&a->stage_rays, 2 * want * 8 * sizeof(float)));
        LMGPU_CUDA_TRY(cudaMalloc((void**)&a->stage_hits, 2 * want * sizeof(lmgpu_hit)));
        a->stage_cap = want;
    }
    for (int i = 0; i < 2; i++)
        if (!a->stage_stream[i]) LMGPU_CUDA_TRY(cudaStreamCreateWithFlags(&a->stage_stream[i], cudaStreamNonBlocking));
    // Small batches keep the copy/compute pipeline full.
    uint64_t batch = n / 8;
    batch = batch < (1ull << 18) ? (1ull << 18) : batch;
    batch = batch > a->stage_cap ? a->stage_cap : batch;
    int rc = LMGPU_OK;
    cudaError_t e = cudaSuccess;
    uint64_t k = 0;
    for (uint64_t off = 0; off < n; off += batch, k++) {
        const uint64_t m = (n - off) < batch ? (n - off) : batch;
        const int h = (int)(k & 1);
        cudaStream_t s = a->stage_stream[h];
        float* dr = a->stage_rays + (uint64_t)h * a->stage_cap * 8;
        lmgpu_hit* dh = a->stage_hits + (uint64_t)h * a->stage_cap;
        e = cudaMemcpyAsync(dr, rays + 8 * off, m * 8 * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) break;
        rc = launch_trace(a, reinterpret_cast<const float4*>(dr), dh, m, anyhit != 0, false, s);
        if (rc) break;
        e = cudaMemcpyAsync(hits + off, dh, m * sizeof(lmgpu_hit), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) break;
    }
    for (int i = 0; i < 2; i++) {
        cudaError_t e2 = cudaStreamSynchronize(a->stage_stream[i]);
        if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) {
        set_error(std::string("lmgpu_trace: ") + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    if (rc) return rc;
    return read_status(a, a->stage_stream[0]);
}

int lmgpu_accel_set_tuning(lmgpu_accel* a, int refill, int postpone)
{
    clear_error();
    if (!a || refill < 1 || refill > 32 || postpone < 0 || postpone > 32) {
        set_error("lmgpu_accel_set_tuning: refill must be in [1, 32] and postpone in [0, 32]");
        return LMGPU_ERR_INVALID;
    }
    a->tune.refill = refill;
    a->tune.postpone = postpone;
    return LMGPU_OK;
}

int lmgpu_accel_check(const lmgpu_accel* a, void* stream)
{
    clear_error();
    if (!a) {
        set_error("lmgpu_accel_check: NULL accel");
        return LMGPU_ERR_INVALID;
    }
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) {
        set_error(std::string("lmgpu_accel_check: ") + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    return read_status(a, (cudaStream_t)stream);
}

}  // extern "C"
