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

// Byte k of w as a float: the byte becomes the low mantissa bits of 2^23,
// and subtracting 2^23 leaves it exactly (PRMT + FADD instead of a
// shift/mask and an int-to-float conversion).
__device__ __forceinline__ float qbyte(uint32_t w, int k)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (uint32_t)k)) - 8388608.0f;
}

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

// Persistent traversal.  Each block owns the contiguous ray range
// [blockIdx * n / grid, (blockIdx + 1) * n / grid) and its warps take rays
// from it through a shared-memory counter, so no global state outlives a
// launch and concurrent launches on other streams are independent.
//
// Per warp, every iteration of the main loop:
//   1. refill: when at least `refill` lanes are idle, they take new rays
//      together (one shared atomic per warp);
//   2. node step: a lane with no pending triangles visits one node (or pops
//      a group from its stack, or finishes its ray);
//   3. triangle steps: lanes with pending triangles test them one at a time
//      while at least `postpone` lanes of the warp have triangle work; when
//      fewer do, lanes that also have node work push their triangles back on
//      the stack and go on traversing (after Aila & Laine 2009 and Ylitie,
//      Karras & Laine 2017), so the warp keeps doing one kind of work at once.
template <bool ANYHIT, bool STATS>
__global__ void __launch_bounds__(kTraceThreads) k_trace(const WNode* __restrict__ nodes, const WTri* __restrict__ tris,
                                                         const float4* __restrict__ rays, lmgpu_hit* __restrict__ hits,
                                                         uint64_t n, uint32_t num_nodes, uint32_t num_tris,
                                                         int refill, int postpone, uint32_t* __restrict__ status,
                                                         unsigned long long* __restrict__ counters)
{
    __shared__ unsigned long long s_next;
    const uint64_t begin = (uint64_t)blockIdx.x * n / gridDim.x;
    const uint64_t end = (uint64_t)(blockIdx.x + 1) * n / gridDim.x;
    if (threadIdx.x == 0) s_next = begin;
    __syncthreads();
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;

    bool active = false, exhausted = false;
    uint64_t rid = 0;
    RayState R;
    float best_t = 0.0f, best_b1 = 0.0f, best_b2 = 0.0f;
    int best_id = -1;
    uint2 ng = make_uint2(0u, 0u), tg = make_uint2(0u, 0u);
    uint2 stack[kStack];
    int sp = 0;
    uint32_t budget = 0;
    uint32_t node_fetch = 0, tri_fetch = 0, nrays = 0, nhits = 0;

    while (true) {
        // 1. refill idle lanes
        const unsigned idle = __ballot_sync(FULL, !active);
        if (!exhausted && __popc(idle) >= refill) {
            const unsigned leader = __ffs(idle) - 1u;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&s_next, (unsigned long long)__popc(idle));
            base = __shfl_sync(FULL, base, leader);
            if (base + __popc(idle) >= end) exhausted = true;
            if (!active) {
                const uint64_t id = base + __popc(idle & lt_mask);
                if (id < end) {
                    rid = id;
                    const float4 r0 = __ldg(rays + 2 * id);
                    const float4 r1 = __ldg(rays + 2 * id + 1);
                    setup_ray(r0, r1, R);
                    best_t = r1.w;
                    best_id = -1;
                    best_b1 = best_b2 = 0.0f;
                    ng = make_uint2(0u, num_nodes > 0 ? 0x80000000u : 0u);
                    tg = make_uint2(0u, 0u);
                    sp = 0;
                    budget = num_nodes + 1;
                    active = true;
                    if (STATS) nrays++;
                }
            }
        }
        if (!__any_sync(FULL, active)) break;

        // 2. node step
        if (active && tg.y == 0u) {
            if (ng.y & 0xff000000u) {
                const uint32_t bit = 31u - __clz(ng.y & 0xff000000u);
                ng.y &= ~(1u << bit);
                const uint32_t slot = (bit - 24u) ^ R.oct_inv;
                const uint32_t rel = __popc(ng.y & 0xffu & ((1u << slot) - 1u));
                const uint32_t ni = ng.x + rel;
                if (ni >= num_nodes || budget-- == 0u) {
                    atomicOr(status, kStatusBadTree);
                    ng.y = 0u;
                    sp = 0;
                } else {
                    if (ng.y & 0xff000000u) {
                        if (sp < kStack) stack[sp++] = ng;
                        else atomicOr(status, kStatusStackOverflow);
                    }
                    uint32_t child_base, tri_base, imask;
                    const uint32_t hm = intersect_node(nodes, ni, R, best_t, child_base, tri_base, imask);
                    if (STATS) node_fetch++;
                    ng = make_uint2(child_base, (hm & 0xff000000u) | imask);
                    tg = make_uint2(tri_base, hm & 0x00ffffffu);
                }
            } else if (sp > 0) {
                const uint2 g = stack[--sp];
                if (g.y & 0xff000000u) ng = g;
                else tg = g;
            } else {
                lmgpu_hit h;
                h.t = best_id >= 0 ? best_t : 0.0f;
                h.prim = best_id;
                h.b1 = best_b1;
                h.b2 = best_b2;
                reinterpret_cast<float4*>(hits)[rid] = *reinterpret_cast<const float4*>(&h);
                if (STATS && best_id >= 0) nhits++;
                active = false;
            }
        }

        // 3. triangle steps
        while (true) {
            const bool has = active && tg.y != 0u;
            const unsigned m = __ballot_sync(FULL, has);
            if (m == 0u) break;
            const bool few = __popc(m) < postpone;
            if (few && has && (ng.y & 0xff000000u) && sp < kStack) {
                stack[sp++] = tg;
                tg.y = 0u;
            }
            if (active && tg.y != 0u) {
                const uint32_t k = __ffs(tg.y) - 1u;
                tg.y &= tg.y - 1u;
                if (tg.x + k >= num_tris) {
                    atomicOr(status, kStatusBadTree);
                    tg.y = 0u;
                } else {
                    float t, b1, b2;
                    int id;
                    if (STATS) tri_fetch++;
                    if (intersect_tri(tris, tg.x + k, R, best_t, t, b1, b2, id)) {
                        if (t < best_t || id > best_id) {
                            best_t = t;
                            best_id = id;
                            best_b1 = b1;
                            best_b2 = b2;
                        }
                        if (ANYHIT) {
                            tg.y = 0u;
                            ng.y = 0u;
                            sp = 0;
                        }
                    }
                }
            }
            if (few) break;
        }
    }
    if (STATS) {
        unsigned long long v[4] = {nrays, node_fetch, tri_fetch, nhits};
        for (int q = 0; q < 4; q++) {
            unsigned long long x = v[q];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULL, x, o);
            if (lane == 0) atomicAdd(&counters[q], x);
        }
    }
}

}  // namespace

int launch_trace(const lmgpu_accel* a, const float4* d_rays, lmgpu_hit* d_hits, uint64_t n, bool anyhit, bool stats,
                 cudaStream_t stream)
{
    if (n == 0) return LMGPU_OK;
    static int grid_cap = 0;
    if (grid_cap == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        LMGPU_CUDA_TRY(cudaGetDevice(&dev));
        LMGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        LMGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<false, false>, kTraceThreads, 0));
        grid_cap = sms * (per_sm > 0 ? per_sm : 1);
    }
    const TraceConfig cfg = a->tune;
    // at least ~4 warps' worth of rays per block
    const uint64_t by_rays = (n + 4 * kTraceThreads - 1) / (4 * kTraceThreads);
    const unsigned grid = (unsigned)(by_rays < (uint64_t)grid_cap ? by_rays : (uint64_t)grid_cap);
    const uint32_t nn = a->ntri > 0 ? (uint32_t)a->num_wide : 0u;
    const uint32_t nt = (uint32_t)a->ntri;
    auto* cnt = a->counters;
    if (anyhit) {
        if (stats) k_trace<true, true><<<grid, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, cfg.refill, cfg.postpone, a->status, cnt);
        else k_trace<true, false><<<grid, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, cfg.refill, cfg.postpone, a->status, cnt);
    } else {
        if (stats) k_trace<false, true><<<grid, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, cfg.refill, cfg.postpone, a->status, cnt);
        else k_trace<false, false><<<grid, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, cfg.refill, cfg.postpone, a->status, cnt);
    }
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

}  // namespace lmgpu
