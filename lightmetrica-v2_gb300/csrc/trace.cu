// Ray traversal of the 8-wide compressed BVH (sm_103a).
//
// Replaces the per-ray Accel3::Intersect of the reference
// (include/lightmetrica/accel3.h:68; e.g. accel_bvh_sahbin.cpp:234-288,
// accel_qbvh.cpp:398-497) with a batch kernel, one thread per ray:
//
//   * node groups (child base index + 8-bit hit mask + the node's inner mask)
//     live in a short per-thread stack; the next child is the highest set hit
//     bit, and hit bits of inner children are permuted by the ray octant so
//     that this visits children roughly front to back (the build stores
//     children in octant slots);
//   * each 80-byte node is fetched as five 16-byte read-only loads, and all
//     eight child boxes are tested with one FMA per slab
//     (t = q * (2^e / d) + (p - o) / d);
//   * triangles are 48-byte records, tested with the watertight algorithm of
//     Woop, Benthin and Wald (JCGT 2013): shear to ray space, edge functions
//     with unfused products (so shared edges give exactly negated values),
//     FP64 recomputation when an edge function is exactly zero;
//   * ties at equal t resolve to the higher global triangle id, the outcome
//     of accel::naive's ascending scan with "t > maxT" rejection
//     (triaccel.h:137, accel_naive.cpp:99-110).
#include "accel.cuh"

namespace lmgpu {
namespace {

constexpr int kStack = 32;
constexpr int kTraceThreads = 128;

struct RayState {
    float ox, oy, oz;
    float tmin;
    float idx, idy, idz;  // 1 / d (zero components replaced by a tiny value)
    uint32_t oct_inv;     // 7 - octant; octant bit set = negative direction
    // watertight setup
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__device__ __forceinline__ float comp(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ float safe_rcp(float d)
{
    const float tiny = 1e-20f;
    return 1.0f / (fabsf(d) > tiny ? d : copysignf(tiny, d));
}

__device__ __forceinline__ void setup_ray(const float4 r0, const float4 r1, RayState& R)
{
    R.ox = r0.x; R.oy = r0.y; R.oz = r0.z; R.tmin = r0.w;
    R.idx = safe_rcp(r1.x); R.idy = safe_rcp(r1.y); R.idz = safe_rcp(r1.z);
    const uint32_t oct = (R.idx < 0.0f ? 1u : 0u) | (R.idy < 0.0f ? 2u : 0u) | (R.idz < 0.0f ? 4u : 0u);
    R.oct_inv = 7u - oct;
    const float ax = fabsf(r1.x), ay = fabsf(r1.y), az = fabsf(r1.z);
    int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dkz = comp(r1.x, r1.y, r1.z, kz);
    if (dkz < 0.0f) { const int t = kx; kx = ky; ky = t; }
    R.kx = kx; R.ky = ky; R.kz = kz;
    R.Sx = comp(r1.x, r1.y, r1.z, kx) / dkz;
    R.Sy = comp(r1.x, r1.y, r1.z, ky) / dkz;
    R.Sz = 1.0f / dkz;
}

__device__ __forceinline__ float qbyte(uint32_t w, int k) { return (float)((w >> (8 * k)) & 0xffu); }

// Tests the eight child boxes of one node; returns the hit mask
// (bits 24..31 inner children in permuted slot order, bits 0..23 triangles).
__device__ __forceinline__ uint32_t intersect_node(const WNode* __restrict__ nodes, uint32_t ni, const RayState& R,
                                                   float tmax, uint32_t& child_base, uint32_t& tri_base,
                                                   uint32_t& imask)
{
    const uint4* np = reinterpret_cast<const uint4*>(nodes + ni);
    const uint4 w0 = __ldg(np + 0);
    const uint4 w1 = __ldg(np + 1);
    const uint4 w2 = __ldg(np + 2);
    const uint4 w3 = __ldg(np + 3);
    const uint4 w4 = __ldg(np + 4);
    const float px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
    const float sx = __uint_as_float((w0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
    imask = w0.w >> 24;
    child_base = w1.x;
    tri_base = w1.y;
    const float ax = sx * R.idx, ay = sy * R.idy, az = sz * R.idz;
    const float bx = (px - R.ox) * R.idx, by = (py - R.oy) * R.idy, bz = (pz - R.oz) * R.idz;
    const bool nx = R.idx < 0.0f, ny = R.idy < 0.0f, nz = R.idz < 0.0f;
    uint32_t hm = 0;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const uint32_t meta4 = half ? w1.w : w1.z;
        const uint32_t lox = half ? w2.y : w2.x, loy = half ? w2.w : w2.z, loz = half ? w3.y : w3.x;
        const uint32_t hix = half ? w3.w : w3.z, hiy = half ? w4.y : w4.x, hiz = half ? w4.w : w4.z;
        const uint32_t nearx = nx ? hix : lox, farx = nx ? lox : hix;
        const uint32_t neary = ny ? hiy : loy, fary = ny ? loy : hiy;
        const uint32_t nearz = nz ? hiz : loz, farz = nz ? loz : hiz;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float tnx = fmaf(qbyte(nearx, k), ax, bx);
            const float tny = fmaf(qbyte(neary, k), ay, by);
            const float tnz = fmaf(qbyte(nearz, k), az, bz);
            const float tfx = fmaf(qbyte(farx, k), ax, bx);
            const float tfy = fmaf(qbyte(fary, k), ay, by);
            const float tfz = fmaf(qbyte(farz, k), az, bz);
            const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, R.tmin));
            const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
            if (tn <= tf) {
                const uint32_t meta = (meta4 >> (8 * k)) & 0xffu;
                uint32_t bit = meta & 0x1fu;
                if (bit >= 24u) bit ^= R.oct_inv;
                hm |= (meta >> 5) << bit;
            }
        }
    }
    return hm;
}

// Watertight ray/triangle test.  Returns true and (t, b1, b2) when the ray
// meets the triangle in [tmin, tmax].
__device__ __forceinline__ bool intersect_tri(const WTri* __restrict__ tris, uint32_t ti, const RayState& R,
                                              float tmax, float& t_out, float& b1_out, float& b2_out, int& id_out)
{
    const float4* tp = reinterpret_cast<const float4*>(tris + ti);
    const float4 v0 = __ldg(tp + 0);
    const float4 v1 = __ldg(tp + 1);
    const float4 v2 = __ldg(tp + 2);
    const float Ax3[3] = {v0.x - R.ox, v0.y - R.oy, v0.z - R.oz};
    const float Bx3[3] = {v1.x - R.ox, v1.y - R.oy, v1.z - R.oz};
    const float Cx3[3] = {v2.x - R.ox, v2.y - R.oy, v2.z - R.oz};
    const float Akx = comp(Ax3[0], Ax3[1], Ax3[2], R.kx), Aky = comp(Ax3[0], Ax3[1], Ax3[2], R.ky),
                Akz = comp(Ax3[0], Ax3[1], Ax3[2], R.kz);
    const float Bkx = comp(Bx3[0], Bx3[1], Bx3[2], R.kx), Bky = comp(Bx3[0], Bx3[1], Bx3[2], R.ky),
                Bkz = comp(Bx3[0], Bx3[1], Bx3[2], R.kz);
    const float Ckx = comp(Cx3[0], Cx3[1], Cx3[2], R.kx), Cky = comp(Cx3[0], Cx3[1], Cx3[2], R.ky),
                Ckz = comp(Cx3[0], Cx3[1], Cx3[2], R.kz);
    const float Ax = fmaf(-R.Sx, Akz, Akx), Ay = fmaf(-R.Sy, Akz, Aky);
    const float Bx = fmaf(-R.Sx, Bkz, Bkx), By = fmaf(-R.Sy, Bkz, Bky);
    const float Cx = fmaf(-R.Sx, Ckz, Ckx), Cy = fmaf(-R.Sy, Ckz, Cky);
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = R.Sz * Akz, Bz = R.Sz * Bkz, Cz = R.Sz * Ckz;
    const float T = fmaf(U, Az, fmaf(V, Bz, W * Cz));
    const float t = __fdiv_rn(T, det);
    if (!(t >= R.tmin && t <= tmax)) return false;
    const float rdet = __frcp_rn(det);
    t_out = t;
    b1_out = V * rdet;
    b2_out = W * rdet;
    id_out = __float_as_int(v0.w);
    return true;
}

template <bool ANYHIT, bool STATS>
__global__ void __launch_bounds__(kTraceThreads) k_trace(const WNode* __restrict__ nodes, const WTri* __restrict__ tris,
                                                         const float4* __restrict__ rays, lmgpu_hit* __restrict__ hits,
                                                         uint64_t n, uint32_t num_nodes, uint32_t num_tris,
                                                         uint32_t* __restrict__ status,
                                                         unsigned long long* __restrict__ counters)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (!STATS && i >= n) return;
    const bool active = i < n;
    const float4 r0 = active ? __ldg(rays + 2 * i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 r1 = active ? __ldg(rays + 2 * i + 1) : make_float4(1.0f, 0.0f, 0.0f, -1.0f);
    RayState R;
    setup_ray(r0, r1, R);
    float best_t = r1.w;
    int best_id = -1;
    float best_b1 = 0.0f, best_b2 = 0.0f;
    uint32_t node_fetch = 0, tri_fetch = 0;

    uint2 stack[kStack];
    int sp = 0;
    // Root group: one inner child at bit 31, base 0, inner mask 0.
    uint2 ng = make_uint2(0u, (num_nodes > 0 && active) ? 0x80000000u : 0u);
    bool done = false;
    // A tree visits each node at most once per ray; more iterations than
    // nodes means a malformed tree: flag it and stop instead of looping.
    uint32_t budget = num_nodes + 1;
    while (!done) {
        if (ng.y & 0xff000000u) {
            const uint32_t bit = 31u - __clz(ng.y & 0xff000000u);
            ng.y &= ~(1u << bit);
            const uint32_t slot = (bit - 24u) ^ R.oct_inv;
            const uint32_t rel = __popc(ng.y & 0xffu & ((1u << slot) - 1u));
            const uint32_t ni = ng.x + rel;
            if (ni >= num_nodes || budget-- == 0) {
                atomicOr(status, kStatusBadTree);
                break;
            }
            if (ng.y & 0xff000000u) {
                if (sp < kStack) stack[sp++] = ng;
                else atomicOr(status, kStatusStackOverflow);
            }
            uint32_t child_base, tri_base, imask;
            const uint32_t hm = intersect_node(nodes, ni, R, best_t, child_base, tri_base, imask);
            if (STATS) node_fetch++;
            ng = make_uint2(child_base, (hm & 0xff000000u) | imask);
            uint32_t tmask = hm & 0x00ffffffu;
            while (tmask) {
                const uint32_t k = __ffs(tmask) - 1;
                tmask &= tmask - 1;
                if (tri_base + k >= num_tris) {
                    atomicOr(status, kStatusBadTree);
                    break;
                }
                float t, b1, b2;
                int id;
                if (STATS) tri_fetch++;
                if (intersect_tri(tris, tri_base + k, R, best_t, t, b1, b2, id)) {
                    if (t < best_t || id > best_id) {
                        best_t = t;
                        best_id = id;
                        best_b1 = b1;
                        best_b2 = b2;
                    }
                    if (ANYHIT) {
                        done = true;
                        break;
                    }
                }
            }
        } else if (sp > 0) {
            ng = stack[--sp];
        } else {
            done = true;
        }
    }
    lmgpu_hit h;
    h.t = best_id >= 0 ? best_t : 0.0f;
    h.prim = best_id;
    h.b1 = best_b1;
    h.b2 = best_b2;
    if (active) reinterpret_cast<float4*>(hits)[i] = *reinterpret_cast<const float4*>(&h);
    if (STATS) {
        // every lane of the warp reaches this point (no early return with STATS)
        unsigned long long v[4] = {active ? 1ull : 0ull, node_fetch, tri_fetch, best_id >= 0 ? 1ull : 0ull};
        for (int q = 0; q < 4; q++) {
            unsigned long long x = v[q];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) == 0) atomicAdd(&counters[q], x);
        }
    }
}

}  // namespace

int launch_trace(const lmgpu_accel* a, const float4* d_rays, lmgpu_hit* d_hits, uint64_t n, bool anyhit, bool stats,
                 cudaStream_t stream)
{
    if (n == 0) return LMGPU_OK;
    const uint64_t blocks = (n + kTraceThreads - 1) / kTraceThreads;
    if (blocks > 0x7fffffffull) {
        set_error("lmgpu_trace: too many rays for one launch");
        return LMGPU_ERR_INVALID;
    }
    const uint32_t nn = a->ntri > 0 ? (uint32_t)a->num_wide : 0u;
    const uint32_t nt = (uint32_t)a->ntri;
    if (anyhit) {
        if (stats) k_trace<true, true><<<(unsigned)blocks, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, a->status, a->counters);
        else k_trace<true, false><<<(unsigned)blocks, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, a->status, a->counters);
    } else {
        if (stats) k_trace<false, true><<<(unsigned)blocks, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, a->status, a->counters);
        else k_trace<false, false><<<(unsigned)blocks, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, a->status, a->counters);
    }
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

}  // namespace lmgpu
