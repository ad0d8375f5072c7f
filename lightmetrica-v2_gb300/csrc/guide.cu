// The guiding network on the 5th-generation tensor cores (tcgen05, sm_103a):
// forward, backward and Adam kernels for the MLP of guide_net.cuh, BF16
// operands with FP32 accumulation in tensor memory.
//
// k_guide_fwd   one CTA per SM, persistent over 128-query tiles, as four
//               independent groups of 4 warps that work on alternate tiles
//               (so one group's MMAs overlap the others' feature encoding
//               and epilogues).  The five weight matrices stay in shared
//               memory (BF16, K-major canonical layout); a group's tile
//               activations ping-pong between its two 64-column
//               shared-memory tiles, which together hold the 128 input
//               features of the first layer;
//               each layer is K/16 MMAs of M = 128 into the group's
//               64-column tensor-memory accumulator, issued by one thread and
//               completed through the group's mbarrier.  The bias enters as
//               one more K = 16 MMA (a ones tile against the bias split into
//               two BF16 terms), so the epilogue is ReLU and BF16 rounding in
//               one conversion per pair; the feature encoding and the
//               epilogue run one row per thread, reading the row with
//               tcgen05.ld.  The raw outputs of a tile are staged in the
//               group's activation tiles (free after the last layer) and
//               leave with one bulk copy.
//               MODE_TRAIN also copies every layer's input tile, as the
//               shared-memory image the MMAs read, to global memory with one
//               bulk copy per layer, and writes the raw outputs, for the
//               backward pass.
// k_guide_bwd   one CTA per SM, persistent over 128-sample tiles, as two
//               independent groups of 4 warps on alternate tiles: the loss
//               gradient of the outputs, then for each layer, from the last,
//               dH = dZ W (M = 128 MMA against W^T kept in shared memory, into
//               the group's own 64 tensor-memory columns) and dW += dZ^T H,
//               an M = 128 MMA (dZ^T's 64 rows padded with zeros) over the
//               tile's 128 samples as K, with dZ^T and H^T MN-major (layer
//               1's 128 inputs as two halves of 64, one N = 64 MMA each);
//               H^T is the forward's stored input tile, brought in by one
//               bulk copy while the previous layer finishes.  The dW
//               accumulators (384 columns, zeroed at the start) are shared by
//               both groups and summed across every tile the CTA processes;
//               the bias gradients are summed from the dZ^T tiles in registers
//               while the MMAs run.  After its last tile each CTA writes its
//               gradient once to its own slice of a partials buffer.
// k_guide_reduce  adds the CTAs' partial gradients into the FP32 gradient.
// k_guide_adam  Adam on the FP32 master parameters (gradients zeroed).
//
// Every mbarrier wait has an iteration limit; on time-out a kernel raises
// kStatusTimeout in its status word, still frees its tensor memory, and
// returns.
#include "common.cuh"
#include "guide_api.cuh"
#include "lmgpu.h"
#include "guide_net.cuh"
#include "tc.cuh"

#include <cuda_bf16.h>
#include <cstring>
#include <vector>

namespace lmgpu {
namespace {

using namespace guide;

constexpr uint32_t kStatusTimeout = 16;
constexpr uint32_t kWaitLimit = 1u << 24;
constexpr int kTile = 128;
constexpr int kThreads = 256;      // backward: two tile groups of 128 threads, one sample each
constexpr int kFwdGroups = 4;      // forward: tile groups of 128 threads, one query each
constexpr int kFwdThreads = 128 * kFwdGroups;
constexpr int kActs = kIn + 4 * kHid;  // stored activations per sample (bf16)
// Stored activations of the training forward, tile by tile: the inputs of
// layers 1..5 of a 128-sample tile as the K-major canonical images the
// forward multiplies (the features as two 16 KB tiles of 64 columns, then
// four 16 KB hidden tiles).  The same bytes are the MN-major H^T operands of
// the backward's weight gradients (MN = 64 each), so both sides move them
// with bulk copies.
constexpr uint32_t kActTileBytes = (uint32_t)kTile * kActs * 2u;  // 98,304
__host__ __device__ constexpr uint32_t act_off(int l)
{
    return l == 0 ? 0u : (uint32_t)kTile * kIn * 2u + (uint32_t)kTile * kHid * 2u * (uint32_t)(l - 1);
}
__host__ __device__ constexpr uint32_t act_bytes(int l) { return (uint32_t)kTile * 2u * (uint32_t)layer_in(l); }

// shared-memory plan of the forward kernel (bytes)
// W1 (64x128) at 0, W2..W4 (64x64) at 16384 + 8192 (l - 1), W5 (48x64) at 40960
__host__ __device__ constexpr uint32_t fwd_w(int l) { return l == 0 ? 0u : 16384u + 8192u * (uint32_t)(l - 1); }
// per tile group two 128 x 64 activation tiles X and Y (K-major, K = 64);
// layer 1's 128 input features are X (0..63) and Y (64..127), and the
// layers then alternate X -> Y -> X ...
__host__ __device__ constexpr uint32_t fwd_x(uint32_t g) { return 47104u + 32768u * g; }
__host__ __device__ constexpr uint32_t fwd_y(uint32_t g) { return fwd_x(g) + 16384u; }
constexpr uint32_t kFwdBar = fwd_x(kFwdGroups);  // two mbarriers per group (MMAs, queries), the TMEM address
// per group the next tile's 128 queries (9 floats each), brought in by one
// bulk copy while the current tile runs
constexpr uint32_t kTileQueryBytes = (uint32_t)kTile * 9u * 4u;  // 4,608
__host__ __device__ constexpr uint32_t fwd_q(uint32_t g) { return kFwdBar + 128u + kTileQueryBytes * g; }
// the bias as one more K = 16 MMA per layer: a constant 128 x 16 tile whose
// columns 0 and 1 are ones, against a per-layer N x 16 tile holding the bias
// split into two BF16 terms (hi + lo, about 16 significant bits)
constexpr uint32_t kFwdOnes = fwd_q(kFwdGroups);                             // 4 KB
__host__ __device__ constexpr uint32_t fwd_bt(int l) { return kFwdOnes + 4096u + 2048u * (uint32_t)l; }  // 2 KB each
constexpr uint32_t kFwdSmem = fwd_bt(5);

// shared-memory plan of the backward kernel (bytes)
// W_l^T for l = 1..4 (W2^T..W4^T 64x64, W5^T 64x48) at 8192 (l - 1), shared by both tile groups
__host__ __device__ constexpr uint32_t bwd_wt(int l) { return 8192u * (uint32_t)(l - 1); }
// per tile group g: dZ (128 samples x 64, K-major, K = layer width), dZ^T (MN-major,
// 128 features of which 64 are used x 128 samples) and H^T (MN-major, up to 128
// features x 128 samples): each thread stores its sample's features 8 at a time
__host__ __device__ constexpr uint32_t bwd_dz(uint32_t g) { return 30720u + 81920u * g; }
__host__ __device__ constexpr uint32_t bwd_dzt(uint32_t g) { return bwd_dz(g) + 16384u; }
__host__ __device__ constexpr uint32_t bwd_ht(uint32_t g) { return bwd_dzt(g) + 32768u; }
constexpr uint32_t kBwdBar = bwd_dz(2);        // two mbarriers per group (MMAs, bulk loads), the TMEM address
constexpr uint32_t kBwdSmem = kBwdBar + 64;    // 194,624 bytes: one CTA per SM, holding all 512 TMEM columns
// tensor-memory columns of the backward kernel: group g's dH at 64 g, layer 1's
// dW at 128 (128 columns), layer l = 1..4's dW at 256 + 64 (l - 1)
__host__ __device__ constexpr uint32_t bwd_dw_col(int l) { return l == 0 ? 128u : 256u + 64u * (uint32_t)(l - 1); }

enum : int { MODE_RAW = 0, MODE_TRAIN = 1 };

struct Box {
    float lo[3], inv_ext[3];
};

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// 8 consecutive values of row r into a K-major canonical tile (one 16-byte store).
__device__ __forceinline__ void put8(unsigned char* tile, uint32_t r, uint32_t k, uint32_t K, const float v[8])
{
    uint4 q;
    q.x = pack2(v[0], v[1]);
    q.y = pack2(v[2], v[3]);
    q.z = pack2(v[4], v[5]);
    q.w = pack2(v[6], v[7]);
    *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(r, k, K)) = q;
}

// Features m .. m + 7 (m a multiple of 8) of sample k into an MN-major tile
// with MN feature rows.
__device__ __forceinline__ void put8mn(unsigned char* tile, uint32_t m, uint32_t k, uint32_t MN, uint4 q)
{
    *reinterpret_cast<uint4*>(tile + tc::mnmajor_offset(m, k, MN)) = q;
}

// W (rows x cols, fp32 row-major; transpose: stored as W^T) into a K-major tile.
__device__ void load_matrix(unsigned char* tile, const float* __restrict__ W, int rows, int cols, bool transpose)
{
    if (!transpose) {
        for (int idx = threadIdx.x; idx < rows * cols / 8; idx += blockDim.x) {
            const int r = idx / (cols / 8), c = (idx % (cols / 8)) * 8;
            float v[8];
            for (int q = 0; q < 8; q++) v[q] = W[r * cols + c + q];
            put8(tile, r, c, cols, v);
        }
    } else {
        // tile rows = W columns (cols of them), tile K = W rows
        for (int idx = threadIdx.x; idx < rows * cols / 8; idx += blockDim.x) {
            const int r = idx / (rows / 8), c = (idx % (rows / 8)) * 8;
            float v[8];
            for (int q = 0; q < 8; q++) v[q] = W[(c + q) * cols + r];
            put8(tile, r, c, rows, v);
        }
    }
}

// Issues one M = 128 layer, the bias MMA (ones x bias tile) and then its
// K / 16 MMAs, and commits them to the mbarrier.  The A operand is K / 64
// tiles of 64 columns (K-major, K = 64): a0 holds columns 0..63, a1 64..127.
__device__ __forceinline__ void issue_layer(uint32_t d_tmem, uint32_t a0, uint32_t a1, uint32_t K, uint32_t b_saddr,
                                            uint32_t N, uint32_t ones_saddr, uint32_t bias_saddr, uint64_t* bar)
{
    const uint32_t idesc = tc::idesc_bf16_f32(128, N);
    tc::mma_bf16(d_tmem, tc::kmajor_desc(ones_saddr, 16u), tc::kmajor_desc(bias_saddr, 16u), idesc, 0u);
    for (uint32_t ks = 0; ks < K / 16; ks++)
        tc::mma_bf16(d_tmem, tc::kmajor_desc((ks < 4u ? a0 : a1) + (ks & 3u) * 256u, 64u),
                     tc::kmajor_desc(b_saddr + ks * 256u, K), idesc, 1u);
    tc::mma_commit(bar);
}

// relu(a), relu(b) rounded to BF16 and packed (a in the low half).
__device__ __forceinline__ uint32_t relu_pack2(float a, float b)
{
    uint32_t r;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
    return r;
}

// Named barrier over the 128 threads of tile group g (barrier 1 + g;
// barrier 0 is __syncthreads).
__device__ __forceinline__ void group_sync(uint32_t g)
{
    asm volatile("bar.sync %0, 128;" ::"r"(1u + g) : "memory");
}

// The same barrier, returning whether every thread of the group passed v.
__device__ __forceinline__ bool group_sync_and(uint32_t g, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(v ? 1u : 0u), "r"(1u + g)
        : "memory");
    return r != 0u;
}

__device__ __forceinline__ void group_sync_for_mma(uint32_t g)
{
    tc::fence_smem_async();
    tc::fence_before_sync();
    group_sync(g);
    tc::fence_after_sync();
}

// All threads of tile group g: wait for the group's committed MMAs (bounded),
// agree on the outcome, then order tensor-memory reads after them.
__device__ __forceinline__ bool group_wait_layer(uint32_t g, uint64_t* bar, uint32_t& phase, uint32_t* status)
{
    const bool mine = tc::mbar_wait(bar, phase, kWaitLimit);
    phase ^= 1u;
    const bool ok = group_sync_and(g, mine);
    if (!ok && (threadIdx.x & 127u) == 0u) atomicOr(status, kStatusTimeout);
    tc::fence_after_sync();
    return ok;
}

template <int MODE>
__global__ void __launch_bounds__(kFwdThreads, 1) k_guide_fwd(const float* __restrict__ params, Box box,
                                                              const float* __restrict__ queries, uint32_t n,
                                                              const uint32_t* __restrict__ d_n,
                                                              float* __restrict__ raw_out,
                                                              __nv_bfloat16* __restrict__ acts,
                                                              uint32_t* __restrict__ status)
{
    if (d_n) n = *d_n;  // query count on the device (at most the n launched for)
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kFwdBar);  // MMA barriers, then query barriers
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(smem + kFwdBar + 16u * kFwdGroups);
    // four independent tile groups of 128 threads, one row of a tile each;
    // group g works on tiles 4 blockIdx.x + g, + 4 gridDim.x, ..., with its
    // own activation buffers, mbarrier and 64 tensor-memory columns, so one
    // group's MMAs run while the others compute features or epilogues.  A
    // warp reads tensor memory lanes 32 (warp % 4) .. + 31, its rows.
    const uint32_t tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, r = tid & (kTile - 1u);
    const uint32_t lane_base = (warp & 3u) * 32u;

    for (int l = 0; l < 5; l++) load_matrix(smem + fwd_w(l), params + w_off(l), layer_out(l), layer_in(l), false);
    // the ones tile and the bias tiles (K-major, K = 16)
    for (uint32_t i = tid; i < (uint32_t)kTile * 16u; i += kFwdThreads) {
        const uint32_t rr = i >> 4, k = i & 15u;
        *reinterpret_cast<__nv_bfloat16*>(smem + kFwdOnes + tc::kmajor_offset(rr, k, 16u)) =
            __float2bfloat16_rn(k < 2u ? 1.0f : 0.0f);
    }
    for (uint32_t i = tid; i < 5u * 64u * 16u; i += kFwdThreads) {
        const int l = (int)(i / 1024u);
        const uint32_t nn = (i >> 4) & 63u, k = i & 15u;
        float v = 0.0f;
        if (nn < (uint32_t)layer_out(l) && k < 2u) {
            const float b = params[b_off(l) + nn];
            const float hi = __bfloat162float(__float2bfloat16_rn(b));
            v = k == 0u ? hi : b - hi;
        }
        if (nn < (uint32_t)layer_out(l))
            *reinterpret_cast<__nv_bfloat16*>(smem + fwd_bt(l) + tc::kmajor_offset(nn, k, 16u)) = __float2bfloat16_rn(v);
    }
    if (tid == 0) {
        for (int i = 0; i < 2 * kFwdGroups; i++) tc::mbar_init(bars + i, 1);
        tc::mbar_init_fence();
    }
    if (warp == 0) tc::tmem_alloc(s_tmem, 256);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *s_tmem + 64u * g;
    uint64_t* bar = bars + g;
    uint64_t* qbar = bars + kFwdGroups + g;
    unsigned char* bufX = smem + fwd_x(g);
    unsigned char* bufY = smem + fwd_y(g);
    const float* sq = reinterpret_cast<const float*>(smem + fwd_q(g));
    const uint32_t sX = tc::smem_addr(bufX), sY = tc::smem_addr(bufY), sQ = tc::smem_addr(smem + fwd_q(g));
    uint32_t phase = 0, qphase = 0;
    bool alive = true, q_pending = false;

    const uint32_t ntiles = (n + kTile - 1) / kTile;
    // full tiles of a 16-byte aligned query array come in by bulk copy, the
    // next one while the current one runs; a partial last tile is read
    // directly (a bulk copy would read past the array)
    const bool q_bulk = ((uintptr_t)queries & 15u) == 0u;
    auto full_tile = [&](uint32_t t) { return q_bulk && (uint64_t)(t + 1) * kTile <= (uint64_t)n; };
    auto fetch_queries = [&](uint32_t t) {
        if (r == 0) {
            tc::mbar_arrive_expect_tx(qbar, kTileQueryBytes);
            tc::bulk_load(sQ, queries + (size_t)t * kTile * 9u, kTileQueryBytes, qbar);
        }
        q_pending = true;
    };
    const uint32_t first = kFwdGroups * blockIdx.x + g, stride = kFwdGroups * gridDim.x;
    if (first < ntiles && full_tile(first)) fetch_queries(first);
    for (uint32_t tile = first; tile < ntiles && alive; tile += stride) {
        const uint32_t row = tile * kTile + r;
        // the previous tile's output copy reads X and Y: done before they
        // are rewritten (the barrier below orders the other threads)
        if (r == 0) tc::bulk_wait_read0();
        // features of the row's query (guide_net.cuh): per axis 16 frequencies
        // (sin, cos), then the normal and the outgoing direction, then zeros;
        // stored eight at a time
        {
            float q9[9];
            if (full_tile(tile)) {
                const bool got = tc::mbar_wait(qbar, qphase, kWaitLimit);
                if (got) {
                    qphase ^= 1u;
                    q_pending = false;
                }
                if (!group_sync_and(g, got)) {
                    if (r == 0) atomicOr(status, kStatusTimeout);
                    alive = false;
                    break;
                }
                for (int j = 0; j < 9; j++) q9[j] = sq[9 * r + j];
            } else {
                group_sync(g);
                for (int j = 0; j < 9; j++) q9[j] = row < n ? queries[9 * (size_t)row + j] : 0.0f;
            }
            // features 0..63 (axes x, y) into X, 64..127 (axis z, normal,
            // direction, zeros) into Y
#pragma unroll
            for (int d = 0; d < 3; d++) {
                float f[32];
                axis_features((q9[d] - box.lo[d]) * box.inv_ext[d], f);
                if (row >= n)
                    for (int j = 0; j < 32; j++) f[j] = 0.0f;
#pragma unroll
                for (int g8 = 0; g8 < 4; g8++)
                    put8(d < 2 ? bufX : bufY, r, (32 * d + 8 * g8) & 63, kHid, f + 8 * g8);
            }
            const float f[8] = {q9[3], q9[4], q9[5], q9[6], q9[7], q9[8], 0.0f, 0.0f};
            const float z8[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            put8(bufY, r, 32, kHid, f);
#pragma unroll
            for (int g8 = 5; g8 < 8; g8++) put8(bufY, r, 8 * g8, kHid, z8);
        }
        group_sync_for_mma(g);
        // the query buffer is free (read before the barrier): the next tile's
        if (tile + stride < ntiles && full_tile(tile + stride)) fetch_queries(tile + stride);
#pragma unroll
        for (int l = 0; l < 5; l++) {
            if (!alive) break;
            // layer 1 reads X and Y, then layers read X, Y, X, Y; outputs
            // go to X, Y, X, Y
            const uint32_t a_in = (l == 0 || (l & 1)) ? sX : sY;
            unsigned char* out_tile = (l & 1) ? bufY : bufX;
            const uint32_t K = layer_in(l), N = layer_out(l);
            if (r == 0) {
                issue_layer(tmem, a_in, sY, K, tc::smem_addr(smem + fwd_w(l)), N, tc::smem_addr(smem + kFwdOnes),
                            tc::smem_addr(smem + fwd_bt(l)), bar);
                if (MODE == MODE_TRAIN) {
                    // the layer's input tiles, as they are, to the stored
                    // activations; their buffers are rewritten only after
                    // the copies have read them
                    unsigned char* dst = reinterpret_cast<unsigned char*>(acts) + (size_t)tile * kActTileBytes + act_off(l);
                    tc::bulk_store(dst, a_in, 16384u);
                    if (l == 0) tc::bulk_store(dst + 16384u, sY, 16384u);
                    tc::bulk_commit();
                    tc::bulk_wait_read0();
                }
            }
            alive = group_wait_layer(g, bar, phase, status);
            if (!alive) break;
            if (l < 4) {
                float h[kHid];
#pragma unroll
                for (int c = 0; c < kHid; c += 16) tc::tmem_load16(tc::tmem_at(tmem, lane_base, c), h + c);
                tc::tmem_wait_ld();
                // the bias is in the accumulator: ReLU and BF16 rounding in one conversion
#pragma unroll
                for (int c = 0; c < kHid; c += 8)
                    *reinterpret_cast<uint4*>(out_tile + tc::kmajor_offset(r, c, kHid)) =
                        make_uint4(relu_pack2(h[c], h[c + 1]), relu_pack2(h[c + 2], h[c + 3]),
                                   relu_pack2(h[c + 4], h[c + 5]), relu_pack2(h[c + 6], h[c + 7]));
            } else {
                float z[kOut];
#pragma unroll
                for (int c = 0; c < kOut; c += 16) tc::tmem_load16(tc::tmem_at(tmem, lane_base, c), z + c);
                tc::tmem_wait_ld();
                // the row into the group's activation tiles, free now (160 B
                // rows, as raw_out holds them), for one bulk copy of the tile
                float4* srow = reinterpret_cast<float4*>(bufX + (size_t)r * kOutUsed * 4u);
#pragma unroll
                for (int c = 0; c < kOutUsed; c += 4) srow[c / 4] = make_float4(z[c], z[c + 1], z[c + 2], z[c + 3]);
            }
            group_sync_for_mma(g);
            if (l == 4 && r == 0) {
                const uint32_t rows = n - tile * kTile < (uint32_t)kTile ? n - tile * kTile : (uint32_t)kTile;
                tc::bulk_store(raw_out + (size_t)tile * kTile * kOutUsed, sX, rows * kOutUsed * 4u);
                tc::bulk_commit();
            }
        }
    }
    // after a time-out, one more bounded wait for this group's MMAs and its
    // query copy in flight
    if (!alive) tc::mbar_wait(bar, phase ^ 1u, kWaitLimit);
    if (q_pending) tc::mbar_wait(qbar, qphase, kWaitLimit);
    if (r == 0) tc::bulk_wait0();
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(*s_tmem, 256);
        tc::tmem_relinquish();
    }
}

__global__ void __launch_bounds__(kThreads, 1) k_guide_bwd(const float* __restrict__ params,
                                                           const float* __restrict__ raw,
                                                           const __nv_bfloat16* __restrict__ acts,
                                                           const float* __restrict__ dirs,
                                                           const float* __restrict__ weights, uint32_t n,
                                                           float inv_batch, float* __restrict__ partials,
                                                           float* __restrict__ loss, uint32_t* __restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kBwdBar);  // MMA barriers 0, 1; load barriers 2, 3
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(smem + kBwdBar + 32);
    // two independent tile groups of 128 threads (one sample each) on
    // alternate tiles; they share the weights and the dW accumulators, and
    // each has its own operand tiles, dH columns, mbarriers and named barrier
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u, g = tid >> 7, r = tid & (kTile - 1u);
    const uint32_t lane_base = (warp & 3u) * 32u;
    unsigned char* sDZ = smem + bwd_dz(g);
    unsigned char* sDZT = smem + bwd_dzt(g);
    unsigned char* sHT = smem + bwd_ht(g);
    const uint32_t sHTa = tc::smem_addr(sHT);
    uint64_t* bar = bars + g;
    uint64_t* lbar = bars + 2 + g;  // the bulk loads of H^T
    // W_l^T for l = 2..5 (tile rows = layer inputs, K = layer outputs)
    for (int l = 1; l < 5; l++) load_matrix(smem + bwd_wt(l), params + w_off(l), layer_out(l), layer_in(l), true);
    // dZ^T feature rows 64..127 stay zero (M padding)
    for (uint32_t i = tid; i < 2u * 32768u / 16u; i += kThreads) {
        const uint32_t gg = i / (32768u / 16u), j = i % (32768u / 16u);
        reinterpret_cast<uint4*>(smem + bwd_dzt(gg))[j] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (tid == 0) {
        for (int i = 0; i < 4; i++) tc::mbar_init(bars + i, 1);
        tc::mbar_init_fence();
    }
    if (warp == 0) tc::tmem_alloc(s_tmem, 512);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *s_tmem;
    // zero the dW accumulators (columns 128..511): both groups then only add
    {
        const uint32_t c0 = 128u + 192u * g;
        for (uint32_t c = 0; c < 192u; c += 16u) tc::tmem_store16_zero(tc::tmem_at(tmem, lane_base, c0 + c));
        tc::tmem_wait_st();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t dh_col = 64u * g;
    uint32_t phase = 0, lphase = 0;
    bool alive = true, load_pending = false;
    float lsum = 0.0f;
    // bias-gradient partial sums: thread r adds features 8 q .. 8 q + 7 (q = r / 16)
    // of samples r % 16 + 16 j, j = 0..7, of every tile, per layer
    float bacc[5][8];
    for (int l = 0; l < 5; l++)
        for (int j = 0; j < 8; j++) bacc[l][j] = 0.0f;
    const uint32_t bq = r >> 4, bk = r & 15u;

    const uint32_t ntiles = (n + kTile - 1) / kTile;
    for (uint32_t tile = 2u * blockIdx.x + g; tile < ntiles && alive; tile += 2u * gridDim.x) {
        const uint32_t row = tile * kTile + r;
        const bool valid = row < n;
        const unsigned char* tacts = reinterpret_cast<const unsigned char*>(acts) + (size_t)tile * kActTileBytes;
        // the last layer's input tile (H_4^T) while the loss gradient is computed
        if (r == 0) {
            tc::mbar_arrive_expect_tx(lbar, act_bytes(4));
            tc::bulk_load(sHTa, tacts + act_off(4), act_bytes(4), lbar);
        }
        load_pending = true;
        // dL/dz of the output layer (rows 40..47 and invalid samples are zero)
        float dz[kHid];
        for (int c = 0; c < kHid; c++) dz[c] = 0.0f;
        if (valid) {
            float z[kOutUsed];
            const float4* zr = reinterpret_cast<const float4*>(raw + (size_t)row * kOutUsed);
            for (int c = 0; c < kOutUsed; c += 4) {
                const float4 v = zr[c / 4];
                z[c] = v.x;
                z[c + 1] = v.y;
                z[c + 2] = v.z;
                z[c + 3] = v.w;
            }
            Lobes L;
            lobes_from_raw(z, L);
            const float w3[3] = {dirs[3 * (size_t)row], dirs[3 * (size_t)row + 1], dirs[3 * (size_t)row + 2]};
            lsum += loss_grad(L, w3, weights[row] * inv_batch, dz);
        }
        // layers 5..1 (l = 4..0), unrolled so that every layer's widths are
        // compile-time constants (register-resident dZ / dH rows)
#pragma unroll
        for (int l = 4; l >= 0; l--) {
            if (!alive) break;
            const uint32_t Nl = layer_out(l), Kin = layer_in(l);
            if (l > 0)
                for (uint32_t c = 0; c < Nl; c += 8) put8(sDZ, r, c, Nl, dz + c);
            // dZ^T (MN = output features, K = samples): this sample's column,
            // eight features per store
            for (uint32_t c = 0; c < (uint32_t)kHid; c += 8)
                put8mn(sDZT, c, r, kTile,
                       make_uint4(pack2(dz[c], dz[c + 1]), pack2(dz[c + 2], dz[c + 3]), pack2(dz[c + 4], dz[c + 5]),
                                  pack2(dz[c + 6], dz[c + 7])));
            // the layer's input H^T (MN = inputs, K = samples) has arrived
            const bool loaded = tc::mbar_wait(lbar, lphase, kWaitLimit);
            if (loaded) {
                lphase ^= 1u;
                load_pending = false;
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            const bool ok = group_sync_and(g, loaded);
            tc::fence_after_sync();
            if (!ok) {
                if (r == 0) atomicOr(status, kStatusTimeout);
                alive = false;
                break;
            }
            if (r == 0) {
                // dW += dZ^T (128 x 128 samples) x (H^T, Kin x 128 samples)^T, in
                // tensor memory across the CTA's tiles; one K step = 16 samples
                // (layer 1's 128 inputs are two MN-major halves of 64, as the
                // forward stored them: one N = 64 MMA per half)
                const uint32_t idesc_w = tc::idesc_bf16_f32_mn(128, 64);
                const uint32_t a0 = tc::smem_addr(sDZT);
                for (uint32_t h = 0; h < Kin / 64u; h++)
                    for (uint32_t ks = 0; ks < (uint32_t)kTile / 16u; ks++)
                        tc::mma_bf16(tmem + bwd_dw_col(l) + 64u * h,
                                     tc::mnmajor_desc(a0 + ks * 2u * (kTile * 16u), kTile),
                                     tc::mnmajor_desc(sHTa + 16384u * h + ks * 2u * (64u * 16u), 64u), idesc_w, 1u);
                // dH_{l-1} = dZ_l (128 x Nl) x (W_l^T, Kin x Nl)^T
                if (l > 0) {
                    const uint32_t idesc_h = tc::idesc_bf16_f32(128, Kin);
                    const uint32_t a1 = tc::smem_addr(sDZ), b1 = tc::smem_addr(smem + bwd_wt(l));
                    for (uint32_t ks = 0; ks < Nl / 16; ks++)
                        tc::mma_bf16(tmem + dh_col, tc::kmajor_desc(a1 + ks * 256u, Nl),
                                     tc::kmajor_desc(b1 + ks * 256u, Nl), idesc_h, ks > 0 ? 1u : 0u);
                }
                tc::mma_commit(bar);
            }
            // while the MMAs run: this thread's share of the bias gradient, the
            // sums over samples of the dZ^T just stored (rows 0..63), and the
            // sample's own input row (the ReLU mask of dZ_{l-1})
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const uint4 v = *reinterpret_cast<const uint4*>(sDZT + tc::mnmajor_offset(8u * bq, bk + 16u * j, kTile));
                const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w4[e]));
                    bacc[l][2 * e] += f.x;
                    bacc[l][2 * e + 1] += f.y;
                }
            }
            uint4 hv[kHid / 8];
            if (l > 0) {
                for (uint32_t q = 0; q < (uint32_t)kHid / 8; q++)
                    hv[q] = *reinterpret_cast<const uint4*>(sHT + tc::kmajor_offset(r, 8u * q, Kin));
                // these reads come before the next bulk load rewrites H^T
                tc::fence_smem_async();
            }
            alive = group_wait_layer(g, bar, phase, status);
            if (!alive) break;
            if (l > 0) {
                // the next layer's input tile, while dZ_{l-1} is formed
                if (r == 0) {
                    tc::mbar_arrive_expect_tx(lbar, act_bytes(l - 1));
                    tc::bulk_load(sHTa, tacts + act_off(l - 1), act_bytes(l - 1), lbar);
                }
                load_pending = true;
                // dZ_{l-1} = dH_{l-1} * relu'(H_{l-1}); H_{l-1} is this layer's input
                float dh[kHid];
                for (int c = 0; c < kHid; c += 16) tc::tmem_load16(tc::tmem_at(tmem, lane_base, dh_col + c), dh + c);
                tc::tmem_wait_ld();
                for (uint32_t q = 0; q < (uint32_t)kHid / 8; q++) {
                    const uint32_t w4[4] = {hv[q].x, hv[q].y, hv[q].z, hv[q].w};
                    for (int e = 0; e < 4; e++) {
                        const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w4[e]));
                        dz[8 * q + 2 * e] = f.x > 0.0f ? dh[8 * q + 2 * e] : 0.0f;
                        dz[8 * q + 2 * e + 1] = f.y > 0.0f ? dh[8 * q + 2 * e + 1] : 0.0f;
                    }
                }
            }
            tc::fence_before_sync();
            group_sync(g);
            tc::fence_after_sync();
        }
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0u && lsum != 0.0f) atomicAdd(loss, lsum);
    // after a time-out, one more bounded wait for this group's MMAs and its
    // bulk load in flight
    if (!alive) {
        tc::mbar_wait(bar, phase ^ 1u, kWaitLimit);
        if (load_pending) tc::mbar_wait(lbar, lphase, kWaitLimit);
    }
    tc::fence_before_sync();
    const bool all_alive = __syncthreads_and(alive ? 1 : 0) != 0;
    tc::fence_after_sync();
    // flush: this CTA's gradient into its slice of the partials.  Bias sums:
    // the 16 threads of a feature group in each tile group, through shared
    // memory (the operand tiles are free now)
    float* part = partials + (size_t)blockIdx.x * kNumParams;
    float* sred = reinterpret_cast<float*>(smem + bwd_dz(0));  // [256 threads][41] (41: no bank conflicts)
    if (all_alive) {
        for (int l = 0; l < 5; l++)
            for (int j = 0; j < 8; j++) sred[tid * 41 + l * 8 + j] = bacc[l][j];
        __syncthreads();
        for (uint32_t i = tid; i < 5u * (uint32_t)kHid; i += kThreads) {
            const uint32_t l = i / kHid, f = i % kHid, q = f >> 3, j = f & 7u;
            float sum = 0.0f;
            for (uint32_t gg = 0; gg < 2; gg++)
                for (uint32_t k = 0; k < 16; k++) sum += sred[(128u * gg + 16u * q + k) * 41u + l * 8u + j];
            if (f < (uint32_t)layer_out(l)) part[b_off(l) + f] = sum;
        }
        // weights: TMEM lanes 0..63 = output features (warps 0 and 1)
        for (int l = 0; l < 5; l++) {
            const uint32_t Kin = layer_in(l);
            if (warp < 2) {
                const uint32_t o = warp * 32 + lane;
                for (uint32_t c = 0; c < Kin; c += 16) {
                    float v[16];
                    tc::tmem_load16(tc::tmem_at(tmem, warp * 32, bwd_dw_col(l) + c), v);
                    tc::tmem_wait_ld();
                    if (o < (uint32_t)layer_out(l))
                        for (int q = 0; q < 16; q++) part[w_off(l) + o * Kin + c + q] = v[q];
                }
            }
        }
    } else {
        for (int i = tid; i < kNumParams; i += kThreads) part[i] = 0.0f;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 512);
        tc::tmem_relinquish();
    }
}

// grad[i] += the CTAs' partial gradients of parameter i.
__global__ void k_guide_reduce(const float* __restrict__ partials, int nparts, float* __restrict__ grad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumParams) return;
    float s = 0.0f;
    for (int b = 0; b < nparts; b++) s += partials[(size_t)b * kNumParams + i];
    grad[i] += s;
}

__global__ void k_guide_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                             float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    g[i] = 0.0f;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace
}  // namespace lmgpu

using namespace lmgpu;

struct lmgpu_guide {
    float* params = nullptr;  // FP32 master parameters
    float* grad = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* loss = nullptr;    // [1]
    uint32_t* status = nullptr;
    Box box{};
    uint64_t step = 0;
    // scratch of the host-pointer entry points and of training
    uint64_t cap = 0;
    float* d_q = nullptr;
    float* d_raw = nullptr;
    float* d_dir = nullptr;
    float* d_w = nullptr;
    __nv_bfloat16* d_acts = nullptr;
    int grid = 0;         // backward: one CTA per SM
    int fwd_grid = 0;     // forward: one CTA (four tile groups) per SM
    float* partials = nullptr;  // [grid][kNumParams] per-CTA gradients of the backward
};

namespace lmgpu {
namespace {

int ensure_scratch(lmgpu_guide* g, uint64_t n)
{
    if (g->cap >= n) return LMGPU_OK;
    void* ptrs[] = {g->d_q, g->d_raw, g->d_dir, g->d_w, g->d_acts};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    g->d_q = g->d_raw = g->d_dir = g->d_w = nullptr;
    g->d_acts = nullptr;
    g->cap = 0;
    if (cudaMalloc(&g->d_q, sizeof(float) * 9 * n) != cudaSuccess ||
        cudaMalloc(&g->d_raw, sizeof(float) * kOutUsed * n) != cudaSuccess ||
        cudaMalloc(&g->d_dir, sizeof(float) * 3 * n) != cudaSuccess ||
        cudaMalloc(&g->d_w, sizeof(float) * n) != cudaSuccess ||
        cudaMalloc(&g->d_acts, (size_t)kActTileBytes * ((n + kTile - 1) / kTile)) != cudaSuccess) {
        set_error("lmgpu_guide: scratch allocation failed");
        return LMGPU_ERR_CUDA;
    }
    g->cap = n;
    return LMGPU_OK;
}

int guide_grid(lmgpu_guide* g)
{
    if (g->grid == 0) {
        int dev = 0, sms = 0;
        LMGPU_CUDA_TRY(cudaGetDevice(&dev));
        LMGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        LMGPU_CUDA_TRY(cudaFuncSetAttribute(k_guide_fwd<MODE_RAW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kFwdSmem));
        LMGPU_CUDA_TRY(cudaFuncSetAttribute(k_guide_fwd<MODE_TRAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kFwdSmem));
        LMGPU_CUDA_TRY(
            cudaFuncSetAttribute(k_guide_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem));
        LMGPU_CUDA_TRY(cudaMalloc((void**)&g->partials, sizeof(float) * (size_t)sms * kNumParams));
        g->grid = sms;
        g->fwd_grid = sms;
    }
    return LMGPU_OK;
}

unsigned tiles_grid(uint64_t n, int cap)
{
    const uint64_t tiles = (n + kTile - 1) / kTile;
    return (unsigned)(tiles < (uint64_t)cap ? tiles : (uint64_t)cap);
}

// Forward CTAs take four tiles at a time, backward CTAs two.
unsigned fwd_grid_of(uint64_t n, int cap) { return tiles_grid((n + kTile - 1) / kTile * (kTile / kFwdGroups), cap); }
unsigned bwd_grid_of(uint64_t n, int cap) { return tiles_grid((n + kTile - 1) / kTile * (kTile / 2), cap); }

int check_status(lmgpu_guide* g, cudaStream_t s, const char* name)
{
    uint32_t st = 0;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&st, g->status, sizeof(st), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (st) {
        set_error(std::string(name) + ": tensor-core wait timed out (status " + std::to_string(st) + ")");
        return LMGPU_ERR_OVERFLOW;
    }
    return LMGPU_OK;
}

}  // namespace

// Device-buffer forward of the raw outputs, used by the guided renderer.
int guide_forward_device(lmgpu_guide* g, const float* d_queries, uint64_t n, float* d_raw, cudaStream_t s)
{
    if (n == 0) return LMGPU_OK;
    int rc = guide_grid(g);
    if (rc) return rc;
    k_guide_fwd<MODE_RAW><<<fwd_grid_of(n, g->fwd_grid), kFwdThreads, kFwdSmem, s>>>(g->params, g->box, d_queries, (uint32_t)n,
                                                                      nullptr, d_raw, nullptr, g->status);
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

// As guide_forward_device with the query count read from d_n on the device
// (at most max_n), so the launch needs no host round trip.
int guide_forward_device_dn(lmgpu_guide* g, const float* d_queries, const uint32_t* d_n, uint64_t max_n,
                            float* d_raw, cudaStream_t s)
{
    if (max_n == 0) return LMGPU_OK;
    int rc = guide_grid(g);
    if (rc) return rc;
    k_guide_fwd<MODE_RAW><<<fwd_grid_of(max_n, g->fwd_grid), kFwdThreads, kFwdSmem, s>>>(g->params, g->box, d_queries,
                                                                          (uint32_t)max_n, d_n, d_raw, nullptr,
                                                                          g->status);
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

// Forward (training) + backward into g->grad for n device samples; the
// mean loss is accumulated into g->loss.
int guide_gradient_device(lmgpu_guide* g, const float* d_queries, const float* d_dirs, const float* d_weights,
                          uint64_t n, cudaStream_t s)
{
    if (n == 0) return LMGPU_OK;
    int rc = guide_grid(g);
    if (rc || (rc = ensure_scratch(g, n))) return rc;
    k_guide_fwd<MODE_TRAIN><<<fwd_grid_of(n, g->fwd_grid), kFwdThreads, kFwdSmem, s>>>(g->params, g->box, d_queries, (uint32_t)n,
                                                                        nullptr, g->d_raw, g->d_acts, g->status);
    LMGPU_CUDA_TRY(cudaGetLastError());
    const unsigned bgrid = bwd_grid_of(n, g->grid);
    k_guide_bwd<<<bgrid, kThreads, kBwdSmem, s>>>(g->params, g->d_raw, g->d_acts, d_dirs, d_weights, (uint32_t)n,
                                                  1.0f / (float)n, g->partials, g->loss, g->status);
    LMGPU_CUDA_TRY(cudaGetLastError());
    k_guide_reduce<<<(kNumParams + 255) / 256, 256, 0, s>>>(g->partials, (int)bgrid, g->grad);
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

void guide_box(const lmgpu_guide* g, float lo[3], float inv_ext[3])
{
    for (int d = 0; d < 3; d++) {
        lo[d] = g->box.lo[d];
        inv_ext[d] = g->box.inv_ext[d];
    }
}

int guide_take_loss(lmgpu_guide* g, cudaStream_t s, float* loss)
{
    float l = 0.0f;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&l, g->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaMemsetAsync(g->loss, 0, sizeof(float), s));
    int rc = check_status(g, s, "lmgpu_guide");
    if (loss) *loss = l;
    return rc;
}

int guide_adam_device(lmgpu_guide* g, float lr, cudaStream_t s)
{
    g->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)g->step), c2 = 1.0f - powf(b2, (float)g->step);
    k_guide_adam<<<(kNumParams + 255) / 256, 256, 0, s>>>(g->params, g->grad, g->m, g->v, kNumParams, lr, b1, b2,
                                                          1e-8f, c1, c2);
    LMGPU_CUDA_TRY(cudaGetLastError());
    return LMGPU_OK;
}

}  // namespace lmgpu

extern "C" {

int lmgpu_guide_num_params(uint64_t* n)
{
    clear_error();
    if (!n) {
        set_error("lmgpu_guide_num_params: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    *n = kNumParams;
    return LMGPU_OK;
}

int lmgpu_guide_create(const float* box_lo_hi, uint32_t seed, lmgpu_guide** out)
{
    clear_error();
    if (!box_lo_hi || !out) {
        set_error("lmgpu_guide_create: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    *out = nullptr;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
        set_error("lmgpu_guide_create: no CUDA device");
        return LMGPU_ERR_NO_DEVICE;
    }
    lmgpu_guide* g = new lmgpu_guide();
    for (int d = 0; d < 3; d++) {
        const float ext = box_lo_hi[3 + d] - box_lo_hi[d];
        g->box.lo[d] = box_lo_hi[d];
        g->box.inv_ext[d] = ext > 0.0f ? 1.0f / ext : 1.0f;
    }
    // He-uniform initial weights from a seeded generator, zero biases;
    // layer-5 padding rows stay zero
    std::vector<float> p(kNumParams, 0.0f);
    uint64_t st = 0x9E3779B97F4A7C15ull ^ seed;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (float)(z >> 40) * (1.0f / 16777216.0f);
    };
    for (int l = 0; l < 5; l++) {
        const int fan_in = l == 0 ? 6 * kFreqs + 6 : kHid;
        const float lim = sqrtf(6.0f / (float)fan_in) * (l == 4 ? 0.1f : 1.0f);
        const int rows = l == 4 ? kOutUsed : layer_out(l);
        for (int o = 0; o < rows; o++)
            for (int i = 0; i < layer_in(l); i++) p[w_off(l) + o * layer_in(l) + i] = (2.0f * next() - 1.0f) * lim;
    }
    const size_t bytes = sizeof(float) * kNumParams;
    if (cudaMalloc(&g->params, bytes) != cudaSuccess || cudaMalloc(&g->grad, bytes) != cudaSuccess ||
        cudaMalloc(&g->m, bytes) != cudaSuccess || cudaMalloc(&g->v, bytes) != cudaSuccess ||
        cudaMalloc(&g->loss, sizeof(float)) != cudaSuccess || cudaMalloc(&g->status, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemcpy(g->params, p.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(g->grad, 0, bytes) != cudaSuccess || cudaMemset(g->m, 0, bytes) != cudaSuccess ||
        cudaMemset(g->v, 0, bytes) != cudaSuccess || cudaMemset(g->loss, 0, sizeof(float)) != cudaSuccess ||
        cudaMemset(g->status, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {  // legacy-stream memsets done before use on other streams
        set_error("lmgpu_guide_create: allocation failed");
        lmgpu_guide_destroy(g);
        return LMGPU_ERR_CUDA;
    }
    *out = g;
    return LMGPU_OK;
}

void lmgpu_guide_destroy(lmgpu_guide* g)
{
    if (!g) return;
    cudaDeviceSynchronize();
    void* ptrs[] = {g->params, g->grad, g->m, g->v, g->loss, g->status, g->d_q, g->d_raw, g->d_dir, g->d_w, g->d_acts,
                    g->partials};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete g;
}

int lmgpu_guide_get_params(const lmgpu_guide* g, float* out, uint64_t n)
{
    clear_error();
    if (!g || !out || n != (uint64_t)kNumParams) {
        set_error("lmgpu_guide_get_params: need lmgpu_guide_num_params floats");
        return LMGPU_ERR_INVALID;
    }
    LMGPU_CUDA_TRY(cudaMemcpy(out, g->params, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return LMGPU_OK;
}

int lmgpu_guide_set_params(lmgpu_guide* g, const float* in, uint64_t n)
{
    clear_error();
    if (!g || !in || n != (uint64_t)kNumParams) {
        set_error("lmgpu_guide_set_params: need lmgpu_guide_num_params floats");
        return LMGPU_ERR_INVALID;
    }
    LMGPU_CUDA_TRY(cudaMemcpy(g->params, in, sizeof(float) * n, cudaMemcpyHostToDevice));
    // a pageable copy may return before its DMA ends; later steps may run on
    // non-blocking streams
    LMGPU_CUDA_TRY(cudaDeviceSynchronize());
    return LMGPU_OK;
}

int lmgpu_guide_forward(lmgpu_guide* g, const float* queries, uint64_t n, float* raw)
{
    clear_error();
    if (!g || (n && (!queries || !raw))) {
        set_error("lmgpu_guide_forward: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    int rc = ensure_scratch(g, n);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemcpy(g->d_q, queries, sizeof(float) * 9 * n, cudaMemcpyHostToDevice));
    if ((rc = guide_forward_device(g, g->d_q, n, g->d_raw, 0))) return rc;
    if ((rc = check_status(g, 0, "lmgpu_guide_forward"))) return rc;
    LMGPU_CUDA_TRY(cudaMemcpy(raw, g->d_raw, sizeof(float) * kOutUsed * n, cudaMemcpyDeviceToHost));
    return LMGPU_OK;
}

int lmgpu_guide_gradient(lmgpu_guide* g, const float* queries, const float* dirs, const float* weights, uint64_t n,
                         float* grad, float* loss)
{
    clear_error();
    if (!g || !grad || (n && (!queries || !dirs || !weights))) {
        set_error("lmgpu_guide_gradient: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    int rc = ensure_scratch(g, n);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemcpy(g->d_q, queries, sizeof(float) * 9 * n, cudaMemcpyHostToDevice));
    LMGPU_CUDA_TRY(cudaMemcpy(g->d_dir, dirs, sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
    LMGPU_CUDA_TRY(cudaMemcpy(g->d_w, weights, sizeof(float) * n, cudaMemcpyHostToDevice));
    LMGPU_CUDA_TRY(cudaMemset(g->grad, 0, sizeof(float) * kNumParams));
    LMGPU_CUDA_TRY(cudaMemset(g->loss, 0, sizeof(float)));
    if ((rc = guide_gradient_device(g, g->d_q, g->d_dir, g->d_w, n, 0))) return rc;
    if ((rc = check_status(g, 0, "lmgpu_guide_gradient"))) return rc;
    LMGPU_CUDA_TRY(cudaMemcpy(grad, g->grad, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost));
    if (loss) LMGPU_CUDA_TRY(cudaMemcpy(loss, g->loss, sizeof(float), cudaMemcpyDeviceToHost));
    LMGPU_CUDA_TRY(cudaMemset(g->grad, 0, sizeof(float) * kNumParams));
    // finished before a later step on a non-blocking stream reads the gradient
    LMGPU_CUDA_TRY(cudaDeviceSynchronize());
    return LMGPU_OK;
}

int lmgpu_guide_forward_device(lmgpu_guide* g, const float* d_queries, uint64_t n, float* d_raw, void* stream)
{
    clear_error();
    if (!g || (n && (!d_queries || !d_raw))) {
        set_error("lmgpu_guide_forward_device: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    return guide_forward_device(g, d_queries, n, d_raw, (cudaStream_t)stream);
}

int lmgpu_guide_train_step_device(lmgpu_guide* g, const float* d_queries, const float* d_dirs, const float* d_weights,
                                  uint64_t n, float lr, void* stream)
{
    clear_error();
    if (!g || (n && (!d_queries || !d_dirs || !d_weights))) {
        set_error("lmgpu_guide_train_step_device: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    int rc = guide_gradient_device(g, d_queries, d_dirs, d_weights, n, (cudaStream_t)stream);
    if (rc) return rc;
    return guide_adam_device(g, lr, (cudaStream_t)stream);
}

int lmgpu_guide_train_step(lmgpu_guide* g, const float* queries, const float* dirs, const float* weights, uint64_t n,
                           float lr, float* loss)
{
    clear_error();
    if (!g || (n && (!queries || !dirs || !weights))) {
        set_error("lmgpu_guide_train_step: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    int rc = ensure_scratch(g, n);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemcpy(g->d_q, queries, sizeof(float) * 9 * n, cudaMemcpyHostToDevice));
    LMGPU_CUDA_TRY(cudaMemcpy(g->d_dir, dirs, sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
    LMGPU_CUDA_TRY(cudaMemcpy(g->d_w, weights, sizeof(float) * n, cudaMemcpyHostToDevice));
    LMGPU_CUDA_TRY(cudaMemset(g->loss, 0, sizeof(float)));
    if ((rc = guide_gradient_device(g, g->d_q, g->d_dir, g->d_w, n, 0)) || (rc = guide_adam_device(g, lr, 0)))
        return rc;
    if ((rc = check_status(g, 0, "lmgpu_guide_train_step"))) return rc;
    if (loss) LMGPU_CUDA_TRY(cudaMemcpy(loss, g->loss, sizeof(float), cudaMemcpyDeviceToHost));
    return LMGPU_OK;
}

}  // extern "C"
