// Blackwell tensor-core primitives (sm_100a family, here sm_103a) as inline
// PTX: tcgen05.mma with FP32 accumulators in tensor memory (TMEM), operands
// in shared memory described by 64-bit matrix descriptors, completion
// tracked by an mbarrier through tcgen05.commit, and tcgen05.ld to bring
// accumulators back to registers.  Written from the PTX ISA's description of
// the tcgen05 instructions, the shared-memory matrix descriptor and the
// kind::f16 instruction descriptor.
//
// Conventions used by the callers:
//   * cta_group::1 (one SM per tile), M = 128: accumulator row m is TMEM
//     lane m, column n is TMEM column n (32-bit cells).  Warp w of the block
//     may read lanes 32 (w % 4) .. 32 (w % 4) + 31 only.
//   * Operands are K-major without swizzling: 8 x 8 BF16 "core matrices"
//     (8 rows of 16 contiguous bytes = 128 contiguous bytes); core matrices
//     adjacent along K are `lbo` bytes apart, groups of 8 rows `sbo` bytes
//     apart.
//   * Every wait on an mbarrier is bounded by wall time (%globaltimer); a
//     wait that runs out returns false and the caller records it.
#pragma once

#include <cstdint>

namespace vsmc_cuda
{
namespace tc05
{

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (K-major: between core matrices adjacent along K), stride byte
// offset (between 8-row groups), the fixed version bits 46-48 = 0b001, no
// base offset, relative LBO mode, no swizzle.
__device__ __forceinline__ uint64_t desc_kmajor(
    uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;
}

// kind::f16 instruction descriptor: D in FP32, A and B in BF16, both
// K-major, dense, shape M x N (M = 64 / 128, N a multiple of 8 / 16).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4)                                  // D: F32
        | (1u << 7)                                   // A: BF16
        | (1u << 10)                                  // B: BF16
        | (static_cast<uint32_t>(N >> 3) << 17)       // N / 8
        | (static_cast<uint32_t>(M >> 4) << 24);      // M / 16
}

// D[tmem] (+)= A[smem] * B[smem]^T over K = 16; accumulate != 0 adds to D.
// Issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc,
    uint64_t b_desc, uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier completes one phase when every tcgen05 operation this thread
// issued before has finished (their shared-memory reads included).
__device__ __forceinline__ void commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one."
                 "shared::cluster.b64 [%0];"
                 :
                 : "r"(smem_addr(mbar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// TMEM columns for the block (one whole warp calls it); the base address is
// written to *dst (shared memory).  ncols: a power of two, 32 .. 512.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 "
                 "[%0], %1;"
                 :
                 : "r"(smem_addr(dst)), "r"(ncols)
                 : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
            : "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :
                 : "r"(taddr), "r"(ncols)
                 : "memory");
}

// 16 consecutive 32-bit columns of this thread's lane (32x32b shape: thread
// t of the warp reads lane base + t).  Followed by wait_ld before use.
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                 "%13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]),
                 "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
                 "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                 "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i)
        v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
                 :
                 : "r"(smem_addr(mbar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait until the phase of the given parity has completed; false after
// `limit_ns` of wall time without it.
__device__ __forceinline__ bool mbar_wait(
    uint64_t *mbar, uint32_t parity, uint64_t limit_ns)
{
    const uint32_t a = smem_addr(mbar);
    const uint64_t t0 = global_ns();
    for (;;) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done)
            return true;
        if (global_ns() - t0 > limit_ns)
            return false;
    }
}

} // namespace tc05
} // namespace vsmc_cuda
