// Shared device/host helpers of the lmgpu library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include <string>

namespace lmgpu {

// ---------------------------------------------------------------------------
// Error reporting: one message per host thread, read by lmgpu_last_error().
void set_error(const std::string& msg);
void clear_error();

#define LMGPU_CUDA_TRY(expr)                                                        \
    do {                                                                            \
        cudaError_t e_ = (expr);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            ::lmgpu::set_error(std::string(#expr) + ": " + cudaGetErrorString(e_)); \
            return LMGPU_ERR_CUDA;                                                  \
        }                                                                           \
    } while (0)

// Status bits raised by kernels into a device word.
enum : uint32_t {
    kStatusStackOverflow = 1u << 0,
    kStatusBuildOverflow = 1u << 1,
    kStatusBadTree = 1u << 2,  // traversal met an out-of-range index or too many nodes
};

// ---------------------------------------------------------------------------
// Ordered-uint encoding of floats, so that atomicMin/atomicMax on uint32
// order like the floats they encode (NaN-free inputs).
__host__ __device__ __forceinline__ uint32_t float_to_ordered(float f)
{
#ifdef __CUDA_ARCH__
    uint32_t u = __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__host__ __device__ __forceinline__ float ordered_to_float(uint32_t u)
{
    uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(v);
#else
    float f;
    memcpy(&f, &v, 4);
    return f;
#endif
}

// Encoded +FLT_MAX / -FLT_MAX, the initial values of min / max reductions.
__host__ __device__ __forceinline__ uint32_t ordered_pos_max() { return 0x80000000u | 0x7f7fffffu; }
__host__ __device__ __forceinline__ uint32_t ordered_neg_max() { return ~(0x80000000u | 0x7f7fffffu); }

// ---------------------------------------------------------------------------
// Device data layouts.

// Binary node of the binned-SAH tree (48 bytes).  Every subtree covers the
// contiguous primitive range [begin, begin + count) of the final index array.
struct BNode {
    float lo[3];
    int32_t left;   // left child (right = left + 1), -1 for a leaf
    float hi[3];
    int32_t begin;
    int32_t count;
    int32_t depth;
    int32_t pad[2];
};
static_assert(sizeof(BNode) == 48, "BNode layout");

// 8-wide compressed node (80 bytes, five 16-byte words).
//   w0: origin p (3 floats), byte exponents ex, ey, ez, inner mask imask
//   w1: child_base, tri_base, leaf mask lmask, 0
//   w2: qlo_x[0..7], qlo_y[0..7]
//   w3: qlo_z[0..7], qhi_x[0..7]
//   w4: qhi_y[0..7], qhi_z[0..7]
// Child box of slot i on axis a: [p_a + qlo_a[i] * 2^e_a, p_a + qhi_a[i] * 2^e_a].
// Slot i holds an inner child (imask bit i: wide node child_base + number of
// inner slots below i), one triangle (lmask bit i: triangle tri_base + number
// of leaf slots below i), or nothing.
struct __align__(16) WNode {
    uint4 w[5];
};
static_assert(sizeof(WNode) == 80, "WNode layout");

// Triangle record (48 bytes): three float4 with the global id in v0.w.
struct __align__(16) WTri {
    float4 v0, v1, v2;
};

// A queue slot for every thread of a kWarps-warp block with take set, with
// one global atomic on *count per block (ordered by warp, then lane);
// threads without take get an unused value.  Every thread of the block must
// call it: it synchronises the block, so it is called only at the top level
// of kernels without early returns; a second call in the same kernel needs a
// __syncthreads() after the first one's slot has been taken.
template <int kWarps>
__device__ __forceinline__ uint32_t block_append_slot(bool take, uint32_t* __restrict__ count)
{
    static_assert(kWarps >= 1 && kWarps <= 32, "one scan warp covers the block");
    __shared__ uint32_t s_off[kWarps];
    const unsigned m = __ballot_sync(0xffffffffu, take);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0u) s_off[warp] = (uint32_t)__popc(m);
    __syncthreads();
    if (warp == 0u) {
        // the warps' counts scanned by warp 0, one atomic for the block's total
        const uint32_t c = lane < (unsigned)kWarps ? s_off[lane] : 0u;
        uint32_t x = c;
#pragma unroll
        for (unsigned o = 1; o < 32u; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, x, 31);
        uint32_t base = 0u;
        if (lane == 0u && tot) base = atomicAdd(count, tot);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (lane < (unsigned)kWarps) s_off[lane] = base + x - c;
    }
    __syncthreads();
    return s_off[warp] + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

}  // namespace lmgpu
