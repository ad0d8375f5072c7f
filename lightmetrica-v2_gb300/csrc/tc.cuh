// 5th-generation tensor core (tcgen05) building blocks for sm_103a, written
// as inline PTX: tensor-memory allocation, shared-memory matrix and
// instruction descriptors, the BF16 MMA with FP32 accumulation in tensor
// memory, its completion through an mbarrier (waited on with an iteration
// limit), and tensor-memory loads for the epilogue.
//
// Operand layouts: "K-major, no swizzle" canonical layout, and its
// MN-major counterpart for operands stored one K index at a time.
// An R x K tile of bf16 is a grid of 8 x 8 core matrices; each core matrix
// is 8 rows of 16 contiguous bytes (128 bytes).  Element (r, k) lives at
//   (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 (core matrices adjacent along K are contiguous) and
// SBO = (K / 8) * 128.  One MMA consumes K = 16 (two core matrices), so the
// descriptors of successive K steps advance by 256 bytes.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace lmgpu {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, k) in a K-major canonical tile with K columns.
__host__ __device__ __forceinline__ uint32_t kmajor_offset(uint32_t r, uint32_t k, uint32_t K)
{
    return (r >> 3) * (K * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// "MN-major, no swizzle" canonical layout of an MN x K tile: each core
// matrix is 8 K-rows of 16 bytes (8 consecutive MN elements); core matrices
// adjacent along MN are contiguous (SBO = 128) and those along K are
// (MN / 8) * 128 bytes apart (LBO).  Element (m, k) lives at
//   (m / 8) * 128 + (k / 8) * (MN / 8) * 128 + (k % 8) * 16 + (m % 8) * 2,
// so eight consecutive MN elements of one K index are one 16-byte store.
__host__ __device__ __forceinline__ uint32_t mnmajor_offset(uint32_t m, uint32_t k, uint32_t MN)
{
    return (m >> 3) * 128u + (k >> 3) * (MN * 16u) + (k & 7u) * 16u + (m & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address, LBO, SBO (bytes, encoded
// >> 4), descriptor version 1 (bits 46-48), base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    return d;
}

// Descriptor of a K-major canonical tile with K columns starting at saddr.
__device__ __forceinline__ uint64_t kmajor_desc(uint32_t saddr, uint32_t K) { return smem_desc(saddr, 128u, K * 16u); }

// Descriptor of an MN-major canonical tile with MN rows starting at saddr
// (LBO = the stride between core matrices along K, SBO = along MN).
__device__ __forceinline__ uint64_t mnmajor_desc(uint32_t saddr, uint32_t MN) { return smem_desc(saddr, MN * 16u, 128u); }

// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major,
// dense, M x N (M = 128: N multiple of 16 in [16, 256]).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// The same with A and B given MN-major (bits 15 and 16: transpose A, B).
__host__ __device__ constexpr uint32_t idesc_bf16_f32_mn(uint32_t M, uint32_t N)
{
    return idesc_bf16_f32(M, N) | (1u << 15) | (1u << 16);
}

// Allocates ncols (power of two, 32..512) tensor-memory columns; the
// address is written to *dst (shared memory).  One full warp executes it.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier at *mbar completes (one arrival) once every tcgen05 operation
// this thread issued before has finished.
__device__ __forceinline__ void mma_commit(uint64_t* mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Generic-proxy shared-memory writes made visible to the tensor core.
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(mbar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

// Makes an mbarrier's initialisation visible to the asynchronous proxy
// (the tensor core's completion arrives through it).
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase with the given parity, at most `limit` polls and at
// most max_ns nanoseconds of wall time; false on time-out (the caller
// records it and winds down).
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit, uint64_t max_ns = 200000000ull)
{
    const uint64_t t0 = global_ns();
    for (uint32_t i = 0; i < limit; i++) {
        if (mbar_test(mbar, parity)) return true;
        if ((i & 255u) == 255u && global_ns() - t0 > max_ns) return false;
    }
    return false;
}

// Bulk (untiled TMA) copies.  Addresses 16-byte aligned, sizes multiples of
// 16 bytes.
// Shared -> global, tracked by bulk groups of the issuing thread.
__device__ __forceinline__ void bulk_store(void* gdst, uint32_t ssrc, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(ssrc), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Until this thread's committed bulk stores have read their shared sources.
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Until they have completed.
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// One arrival on the mbarrier that also expects `bytes` of bulk-copy
// transactions in the current phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bytes)
                 : "memory");
}

// Global -> shared (this CTA), completing `bytes` of transactions on the mbarrier.
__device__ __forceinline__ void bulk_load(uint32_t sdst, const void* gsrc, uint32_t bytes, uint64_t* mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(sdst),
                 "l"(gsrc), "r"(bytes), "r"(smem_addr(mbar))
                 : "memory");
}

// 32 lanes x 16 columns of fp32 from tensor memory: thread i of the warp gets
// lane (taddr.lane + i), columns [taddr.col, taddr.col + 16).
__device__ __forceinline__ void tmem_load16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Zeros 32 lanes x 16 columns of tensor memory (the warp's lanes from taddr.lane).
__device__ __forceinline__ void tmem_store16_zero(uint32_t taddr)
{
    const uint32_t z = 0u;
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1};" ::"r"(taddr),
        "r"(z)
        : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Tensor-memory address of (lane, column).
__device__ __forceinline__ uint32_t tmem_at(uint32_t base, uint32_t lane, uint32_t col)
{
    return base + (lane << 16) + col;
}

}  // namespace tc
}  // namespace lmgpu
