// Device-side ray traversal primitives of the traversal kernel (trace.cu):
// ray set-up, the 8-wide node test and the watertight triangle test.
#pragma once

#include "accel.cuh"

namespace lmgpu {

constexpr int kStack = 32;

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

// Packed FP32 pairs (sm_100 and later): one instruction computes two
// IEEE single-precision results, each rounded as the scalar form would be.
__device__ __forceinline__ unsigned long long pk2(float lo, float hi)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& lo, float& hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

// 2^23 + byte k of w, as a float: the byte becomes the low mantissa bits of
// 2^23 (one PRMT instead of a shift/mask and an int-to-float conversion);
// subtracting 2^23 afterwards leaves the byte exactly.
__device__ __forceinline__ float qbyte23(uint32_t w, int k)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (uint32_t)k));
}

// Slab distances of children k and k + 1 along one axis: q * a + b for the
// two quantised planes q in bytes k, k + 1 of w, as one packed pair.
__device__ __forceinline__ unsigned long long slab2(uint32_t w, int k, unsigned long long a2, unsigned long long b2)
{
    const unsigned long long m2 = 0xCB000000CB000000ull;  // (-2^23, -2^23)
    return fma2(add2(pk2(qbyte23(w, k), qbyte23(w, k + 1)), m2), a2, b2);
}

// Tests the eight child boxes of one node; returns the 8-bit mask of the
// child slots the ray meets, and the node's inner-slot and leaf-slot masks.
// Children are tested in pairs with packed FP32 arithmetic; every distance is
// the same correctly rounded q * a + b as a scalar FMA would give.
__device__ __forceinline__ uint32_t intersect_node(const WNode* __restrict__ nodes, uint32_t ni, const RayState& R,
                                                   float tmax, uint32_t& child_base, uint32_t& tri_base,
                                                   uint32_t& imask, uint32_t& lmask)
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
    lmask = w1.z;
    const float ax = sx * R.idx, ay = sy * R.idy, az = sz * R.idz;
    const float bx = (px - R.ox) * R.idx, by = (py - R.oy) * R.idy, bz = (pz - R.oz) * R.idz;
    const unsigned long long ax2 = pk2(ax, ax), ay2 = pk2(ay, ay), az2 = pk2(az, az);
    const unsigned long long bx2 = pk2(bx, bx), by2 = pk2(by, by), bz2 = pk2(bz, bz);
    const bool nx = R.idx < 0.0f, ny = R.idy < 0.0f, nz = R.idz < 0.0f;
    uint32_t h8 = 0;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const uint32_t lox = half ? w2.y : w2.x, loy = half ? w2.w : w2.z, loz = half ? w3.y : w3.x;
        const uint32_t hix = half ? w3.w : w3.z, hiy = half ? w4.y : w4.x, hiz = half ? w4.w : w4.z;
        const uint32_t nearx = nx ? hix : lox, farx = nx ? lox : hix;
        const uint32_t neary = ny ? hiy : loy, fary = ny ? loy : hiy;
        const uint32_t nearz = nz ? hiz : loz, farz = nz ? loz : hiz;
#pragma unroll
        for (int k = 0; k < 4; k += 2) {
            float tnx[2], tny[2], tnz[2], tfx[2], tfy[2], tfz[2];
            upk2(slab2(nearx, k, ax2, bx2), tnx[0], tnx[1]);
            upk2(slab2(neary, k, ay2, by2), tny[0], tny[1]);
            upk2(slab2(nearz, k, az2, bz2), tnz[0], tnz[1]);
            upk2(slab2(farx, k, ax2, bx2), tfx[0], tfx[1]);
            upk2(slab2(fary, k, ay2, by2), tfy[0], tfy[1]);
            upk2(slab2(farz, k, az2, bz2), tfz[0], tfz[1]);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const float tn = fmaxf(fmaxf(tnx[j], tny[j]), fmaxf(tnz[j], R.tmin));
                const float tf = fminf(fminf(tfx[j], tfy[j]), fminf(tfz[j], tmax));
                // margin 2^-19 relative: above the rounding of both distances
                // (a few ulps of t each, Ize 2013), so a box the ray meets is
                // never rejected although the quantised boxes are tight
                if (tn <= tf * (1.0f + 0x1p-19f)) h8 |= 1u << (4 * half + k + j);
            }
        }
    }
    return h8;
}

// Moves bit s of an 8-bit mask to bit s ^ o (o < 8): inner children in the
// order a ray of octant 7 - o meets them.
__device__ __forceinline__ uint32_t permute_octant(uint32_t h, uint32_t o)
{
    if (o & 1u) h = ((h & 0x55u) << 1) | ((h >> 1) & 0x55u);
    if (o & 2u) h = ((h & 0x33u) << 2) | ((h >> 2) & 0x33u);
    if (o & 4u) h = ((h & 0x0fu) << 4) | ((h >> 4) & 0x0fu);
    return h;
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

}  // namespace lmgpu
