// Surface geometry at hits: the GPU form of
// IntersectionUtils::CreateTriangleIntersection
// (include/lightmetrica/intersectionutils.h:59-135), which every reference
// accel calls on the host for each hit (e.g. accel_bvh_sahbin.cpp:281-285).
// One thread per hit computes, in single precision:
//   p     o + d t (the point the accel passes, accel_naive.cpp:117-121)
//   gn    Normalize(Cross(p2 - p1, p3 - p1))                       :78-82
//   sn    Normalize(n1 (1 - b0 - b1) + n2 b0 + n3 b1), gn when that is NaN
//         or the triangle has no normals                           :84-104
//   uv    uv1 (1 - b0 - b1) + uv2 b0 + uv3 b1, (0, 0) without texcoords
//   dpdu, dpdv   Math::OrthonormalBasis(sn, ...) (math.h:2355-2359)
//   dndu, dndv   (n2 - n1) / |N|, (n3 - n2) / |N| minus their sn components
// and writes each field as planes of n floats (structure of arrays), so
// that a warp's stores are coalesced; the host composes Intersection
// records (ToWorld = (dpdu, dpdv, sn), ToLocal its transpose) from them.
// Products and sums are unfused (explicit round-to-nearest intrinsics) and
// normalisation divides by the correctly rounded length, the generic
// (non-SIMD) form of the reference's Math::Normalize.
#include "accel.cuh"

#include <vector>

namespace lmgpu {
namespace {

constexpr int kSurfaceThreads = 256;

struct F3 {
    float x, y, z;
};

__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 sub3(F3 a, F3 b) { return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ F3 add3(F3 a, F3 b) { return f3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ F3 scl3(F3 a, float s) { return f3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
__device__ __forceinline__ float dot3(F3 a, F3 b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ F3 cross3(F3 a, F3 b)
{
    return f3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y)));
}
__device__ __forceinline__ F3 normalize3(F3 a)
{
    const float l = __fsqrt_rn(dot3(a, a));
    return f3(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}
__device__ __forceinline__ F3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

// One 128-byte record per global triangle, so a hit reads one aligned line
// instead of gathering the triangle (through tri_slot), its normals, its
// texcoords and its flags from four arrays:
//   [0] p1, flags (bit 0 normals, bit 1 texcoords, bit 2 bad slot)
//   [1] p2, n1.x   [2] p3, n1.y   [3] n1.z, n2   [4] n3, uv1.u
//   [5] uv1.v, uv2, uv3.u   [6] uv3.v, 0, 0, 0   [7] unused
constexpr int kSurfRec = 8;  // float4s per record

__global__ void k_surface_pack(const WTri* __restrict__ tris, const int32_t* __restrict__ tri_slot, uint64_t ntri,
                               const float* __restrict__ normals, const float* __restrict__ texcoords,
                               const uint8_t* __restrict__ flags, float4* __restrict__ rec)
{
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ntri) return;
    float4 r[kSurfRec];
    for (int k = 0; k < kSurfRec; k++) r[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t fl = flags ? (uint32_t)(flags[g] & 3u) : 0u;
    const int32_t slot = tri_slot[g];
    if (slot < 0 || (uint64_t)slot >= ntri) {
        fl |= 4u;
    } else {
        const WTri w = tris[slot];
        r[0] = make_float4(w.v0.x, w.v0.y, w.v0.z, 0.0f);
        r[1] = make_float4(w.v1.x, w.v1.y, w.v1.z, 0.0f);
        r[2] = make_float4(w.v2.x, w.v2.y, w.v2.z, 0.0f);
    }
    r[0].w = __uint_as_float(fl);
    if ((fl & 1u) && normals) {
        const float* n = normals + 9 * g;
        r[1].w = n[0];
        r[2].w = n[1];
        r[3] = make_float4(n[2], n[3], n[4], n[5]);
        r[4] = make_float4(n[6], n[7], n[8], 0.0f);
    }
    if ((fl & 2u) && texcoords) {
        const float* t = texcoords + 6 * g;
        r[4].w = t[0];
        r[5] = make_float4(t[1], t[2], t[3], t[4]);
        r[6] = make_float4(t[5], 0.0f, 0.0f, 0.0f);
    }
    for (int k = 0; k < kSurfRec; k++) rec[kSurfRec * g + k] = r[k];
}

__global__ void __launch_bounds__(kSurfaceThreads)
    k_surface(const float4* __restrict__ rec, uint64_t ntri, const float4* __restrict__ rays,
              const lmgpu_hit* __restrict__ hits, uint64_t n, float* __restrict__ out, uint32_t* __restrict__ status)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 hv = reinterpret_cast<const float4*>(hits)[i];
    const int prim = __float_as_int(hv.y);
    float v[23];
    for (int k = 0; k < 23; k++) v[k] = 0.0f;
    if (prim >= 0 && (uint64_t)prim < ntri) {
        const float t = hv.x, b0 = hv.z, b1 = hv.w;
        const float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
        const F3 p = add3(f3(r0.x, r0.y, r0.z), scl3(f3(r1.x, r1.y, r1.z), t));
        const float4* R = rec + (size_t)kSurfRec * prim;
        const float4 ra = R[0], rb = R[1], rc = R[2];
        const uint32_t fl = __float_as_uint(ra.w);
        F3 gn = f3(0.0f, 0.0f, 0.0f), n1 = gn, n2 = gn, n3 = gn, sn = gn;
        if (fl & 4u) {
            atomicOr(status, kStatusBadTree);
        } else {
            const F3 p1 = f3(ra.x, ra.y, ra.z), p2 = f3(rb.x, rb.y, rb.z), p3 = f3(rc.x, rc.y, rc.z);
            gn = normalize3(cross3(sub3(p2, p1), sub3(p3, p1)));
            n1 = n2 = n3 = sn = gn;
        }
        const float w0 = __fsub_rn(__fsub_rn(1.0f, b0), b1);
        float4 re = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (fl & 1u) {
            const float4 rd = R[3];
            re = R[4];
            n1 = f3(rb.w, rc.w, rd.x);
            n2 = f3(rd.y, rd.z, rd.w);
            n3 = f3(re.x, re.y, re.z);
            sn = normalize3(add3(add3(scl3(n1, w0), scl3(n2, b0)), scl3(n3, b1)));
            if (isnan(sn.x) || isnan(sn.y) || isnan(sn.z)) sn = gn;
        }
        float u = 0.0f, uvv = 0.0f;
        if (fl & 2u) {
            if (!(fl & 1u)) re = R[4];
            const float4 rf = R[5], rg = R[6];
            const float tc[6] = {re.w, rf.x, rf.y, rf.z, rf.w, rg.x};
            u = __fadd_rn(__fadd_rn(__fmul_rn(tc[0], w0), __fmul_rn(tc[2], b0)), __fmul_rn(tc[4], b1));
            uvv = __fadd_rn(__fadd_rn(__fmul_rn(tc[1], w0), __fmul_rn(tc[3], b0)), __fmul_rn(tc[5], b1));
        }
        const F3 dpdv = fabsf(sn.x) > fabsf(sn.y) ? normalize3(f3(sn.z, 0.0f, -sn.x)) : normalize3(f3(0.0f, sn.z, -sn.y));
        const F3 dpdu = cross3(dpdv, sn);
        const F3 N = add3(add3(scl3(n1, w0), scl3(n2, b0)), scl3(n3, b1));
        const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(N, N)));
        const F3 dNdu = scl3(sub3(n2, n1), inv), dNdv = scl3(sub3(n3, n2), inv);
        const F3 dndu = sub3(dNdu, scl3(sn, dot3(dNdu, sn)));
        const F3 dndv = sub3(dNdv, scl3(sn, dot3(dNdv, sn)));
        const F3 f[7] = {p, gn, sn, dpdu, dpdv, dndu, dndv};
        for (int k = 0; k < 7; k++) {
            v[3 * k] = f[k].x;
            v[3 * k + 1] = f[k].y;
            v[3 * k + 2] = f[k].z;
        }
        v[21] = u;
        v[22] = uvv;
    }
    for (int k = 0; k < 23; k++) out[(uint64_t)k * n + i] = v[k];
}

// Packs the surface records of the current build (attributes if set).
int pack_surface(lmgpu_accel* a, cudaStream_t stream)
{
    if (a->surf_cap < a->ntri) {
        if (a->surf) cudaFree(a->surf);
        a->surf = nullptr;
        a->surf_cap = 0;
        LMGPU_CUDA_TRY(cudaMalloc((void**)&a->surf, sizeof(float4) * kSurfRec * a->ntri));
        a->surf_cap = a->ntri;
    }
    const bool attrs = a->attr_ntri == a->ntri;
    const uint64_t blocks = (a->ntri + kSurfaceThreads - 1) / kSurfaceThreads;
    k_surface_pack<<<(unsigned)blocks, kSurfaceThreads, 0, stream>>>(
        a->tris, a->tri_slot, a->ntri, attrs ? a->attr_normals : nullptr, attrs ? a->attr_texcoords : nullptr,
        attrs ? a->attr_flags : nullptr, a->surf);
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

int check_surface_args(const lmgpu_accel* a, const char* who)
{
    if (!a->built) {
        set_error(std::string(who) + ": accel not built");
        return LMGPU_ERR_NOT_BUILT;
    }
    return LMGPU_OK;
}

// The records are derived state of the accel, packed on first use after a
// build under the accel's host lock; the wait makes them visible to later
// queries on any stream.  Once packed (surf_ntri published with release
// order after the wait) queries take no lock, so they do not queue behind a
// host trace that holds it.
int ensure_packed(lmgpu_accel* a, cudaStream_t stream)
{
    if (a->ntri == 0 || a->surf_ntri.load(std::memory_order_acquire) == a->ntri) return LMGPU_OK;
    std::lock_guard<std::mutex> lock(a->host_mu);
    if (a->surf_ntri.load(std::memory_order_relaxed) != a->ntri) {
        const int rc = pack_surface(a, stream);
        if (rc) return rc;
        LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
        a->surf_ntri.store(a->ntri, std::memory_order_release);
    }
    return LMGPU_OK;
}

int launch_surface(const lmgpu_accel* ca, const float* d_rays, const lmgpu_hit* d_hits, uint64_t n, float* d_out,
                   cudaStream_t stream)
{
    if (n == 0 || ca->ntri == 0) {
        if (n) LMGPU_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(float) * LMGPU_SURFACE_PLANES * n, stream));
        return LMGPU_OK;
    }
    lmgpu_accel* a = const_cast<lmgpu_accel*>(ca);
    const int rc = ensure_packed(a, stream);
    if (rc) return rc;
    const uint64_t blocks = (n + kSurfaceThreads - 1) / kSurfaceThreads;
    k_surface<<<(unsigned)blocks, kSurfaceThreads, 0, stream>>>(a->surf, a->ntri, reinterpret_cast<const float4*>(d_rays),
                                                                d_hits, n, d_out, a->status);
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

// Waits for stream s and turns the accel's status word into an error.
int surface_status(const lmgpu_accel* a, cudaStream_t s)
{
    uint32_t st = 0;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&st, a->status, sizeof(st), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & kStatusBadTree) {
        set_error("lmgpu_surface: the accel's triangle table is malformed");
        return LMGPU_ERR_OVERFLOW;
    }
    return LMGPU_OK;
}

}  // namespace
}  // namespace lmgpu

using namespace lmgpu;

int lmgpu_accel_set_attributes(lmgpu_accel* a, const float* normals, const float* texcoords, const uint8_t* flags,
                               uint64_t ntri)
{
    clear_error();
    if (!a) {
        set_error("lmgpu_accel_set_attributes: NULL accel");
        return LMGPU_ERR_INVALID;
    }
    if (!a->built) {
        set_error("lmgpu_accel_set_attributes: accel not built");
        return LMGPU_ERR_NOT_BUILT;
    }
    if (ntri != a->ntri) {
        set_error("lmgpu_accel_set_attributes: ntri differs from the built triangle count");
        return LMGPU_ERR_INVALID;
    }
    if (a->attr_normals) cudaFree(a->attr_normals);
    if (a->attr_texcoords) cudaFree(a->attr_texcoords);
    if (a->attr_flags) cudaFree(a->attr_flags);
    a->attr_normals = a->attr_texcoords = nullptr;
    a->attr_flags = nullptr;
    a->attr_ntri = 0;
    a->surf_ntri = 0;
    if (ntri == 0) return LMGPU_OK;
    std::vector<uint8_t> fl(ntri);
    for (uint64_t i = 0; i < ntri; i++)
        fl[i] = flags ? (uint8_t)(flags[i] & 3u) : (uint8_t)((normals ? 1u : 0u) | (texcoords ? 2u : 0u));
    if (normals) {
        LMGPU_CUDA_TRY(cudaMalloc((void**)&a->attr_normals, sizeof(float) * 9 * ntri));
        LMGPU_CUDA_TRY(cudaMemcpy(a->attr_normals, normals, sizeof(float) * 9 * ntri, cudaMemcpyHostToDevice));
    } else {
        for (auto& f : fl) f &= ~1u;
    }
    if (texcoords) {
        LMGPU_CUDA_TRY(cudaMalloc((void**)&a->attr_texcoords, sizeof(float) * 6 * ntri));
        LMGPU_CUDA_TRY(cudaMemcpy(a->attr_texcoords, texcoords, sizeof(float) * 6 * ntri, cudaMemcpyHostToDevice));
    } else {
        for (auto& f : fl) f &= ~2u;
    }
    LMGPU_CUDA_TRY(cudaMalloc((void**)&a->attr_flags, ntri));
    LMGPU_CUDA_TRY(cudaMemcpy(a->attr_flags, fl.data(), ntri, cudaMemcpyHostToDevice));
    a->attr_ntri = ntri;
    int rc = pack_surface(a, nullptr);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaDeviceSynchronize());
    a->surf_ntri.store(ntri, std::memory_order_release);
    return LMGPU_OK;
}

int lmgpu_surface_device(const lmgpu_accel* a, const float* d_rays, const lmgpu_hit* d_hits, uint64_t n,
                         float* d_surface, void* stream)
{
    clear_error();
    if (!a || (n > 0 && (!d_rays || !d_hits || !d_surface))) {
        set_error("lmgpu_surface_device: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    int rc = check_surface_args(a, "lmgpu_surface_device");
    if (rc) return rc;
    return launch_surface(a, d_rays, d_hits, n, d_surface, (cudaStream_t)stream);
}

int lmgpu_surface(const lmgpu_accel* a, const float* rays, const lmgpu_hit* hits, uint64_t n, float* surface)
{
    clear_error();
    if (!a || (n > 0 && (!rays || !hits || !surface))) {
        set_error("lmgpu_surface: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    int rc = check_surface_args(a, "lmgpu_surface");
    if (rc || n == 0) return rc;
    lmgpu_accel* acc = const_cast<lmgpu_accel*>(a);
    cudaStream_t s = 0;
    if ((rc = ensure_packed(acc, s))) return rc;
    // page-locked buffers: the kernel reads the rays and hits and writes the
    // planes across the host link in place
    const void* m_rays = mapped_host(rays);
    const void* m_hits = mapped_host(hits);
    const void* m_out = mapped_host(surface);
    if (m_rays && m_hits && m_out && !(((uintptr_t)m_rays | (uintptr_t)m_hits) & 15u) && !((uintptr_t)m_out & 3u)) {
        rc = launch_surface(a, static_cast<const float*>(m_rays), static_cast<const lmgpu_hit*>(m_hits), n,
                            const_cast<float*>(static_cast<const float*>(m_out)), s);
        if (rc) return rc;
        return surface_status(a, s);
    }
    // pageable buffers: chunks through a staging buffer kept by the accel
    constexpr uint64_t kChunkHits = 1ull << 20;
    constexpr uint64_t kPerHit = 32 + sizeof(lmgpu_hit) + 4 * LMGPU_SURFACE_PLANES;
    std::lock_guard<std::mutex> lock(acc->surf_mu);
    const uint64_t want = n < kChunkHits ? n : kChunkHits;
    if (acc->surf_stage_cap < want) {
        if (acc->surf_stage) cudaFree(acc->surf_stage);
        acc->surf_stage = nullptr;
        acc->surf_stage_cap = 0;
        LMGPU_CUDA_TRY(cudaMalloc((void**)&acc->surf_stage, want * kPerHit));
        acc->surf_stage_cap = want;
    }
    const uint64_t cap = acc->surf_stage_cap;
    float* d_rays = reinterpret_cast<float*>(acc->surf_stage);
    lmgpu_hit* d_hits = reinterpret_cast<lmgpu_hit*>(acc->surf_stage + cap * 32);
    float* d_out = reinterpret_cast<float*>(acc->surf_stage + cap * (32 + sizeof(lmgpu_hit)));
    for (uint64_t off = 0; off < n; off += cap) {
        const uint64_t m = (n - off) < cap ? (n - off) : cap;
        LMGPU_CUDA_TRY(cudaMemcpyAsync(d_rays, rays + 8 * off, m * 32, cudaMemcpyHostToDevice, s));
        LMGPU_CUDA_TRY(cudaMemcpyAsync(d_hits, hits + off, m * sizeof(lmgpu_hit), cudaMemcpyHostToDevice, s));
        if ((rc = launch_surface(a, d_rays, d_hits, m, d_out, s))) return rc;
        // plane k of the chunk -> surface[k n + off ...]
        LMGPU_CUDA_TRY(cudaMemcpy2DAsync(surface + off, n * sizeof(float), d_out, m * sizeof(float),
                                         m * sizeof(float), LMGPU_SURFACE_PLANES, cudaMemcpyDeviceToHost, s));
    }
    return surface_status(a, s);
}
