// Fifth-generation tensor-core primitives (sm_100a / sm_103a): shared-memory matrix descriptors,
// the instruction descriptor of a BF16 x BF16 -> FP32 MMA, Tensor Memory allocation, tcgen05.mma
// with completion on an mbarrier, and tcgen05.ld of the accumulator.  Inline PTX only; every
// wait on an mbarrier is bounded.
//
// Operand layout used here (K-major, no swizzle): a matrix of R rows x K BF16 values is stored as
// 8 x 8 "core matrices" (8 rows of 16 contiguous bytes = 128 bytes).  Core matrix (row group
// rg = r / 8, k group kg = k / 8) starts at rg * SBO + kg * LBO; inside it, row r % 8 starts at
// 16 * (r % 8) and value k % 8 at 2 * (k % 8).  With LBO = 128 the k groups of a row group are
// contiguous and SBO = K * 16.  One MMA consumes K = 16, i.e. two k groups; the next K step starts
// 2 * LBO further.
#ifndef NEIGHBOR_KERNELS_TCGEN05_CUH_
#define NEIGHBOR_KERNELS_TCGEN05_CUH_

#include <cstdint>

#include <cuda_runtime.h>

namespace neighbor
{
namespace gpu
{
namespace tc
{

__device__ __forceinline__ unsigned int smem_addr(const void* p)
    {
    return (unsigned int)__cvta_generic_to_shared(p);
    }

// Byte offset of (row r, value k) in the K-major no-swizzle layout of a matrix with K values
// per row (LBO = 128, SBO = 16 K).
__host__ __device__ constexpr unsigned int kmajor_offset(unsigned int r, unsigned int k, unsigned int K)
    {
    return (r >> 3) * (K * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
    }

// Shared-memory matrix descriptor: start address, leading (K direction) and stride (row
// direction) byte offsets, each >> 4 in 14 bits; bits 46-47 = 1 (the descriptor version of this
// architecture); base offset 0; swizzle mode 0 (none).
__device__ __forceinline__ unsigned long long smem_desc(unsigned int addr, unsigned int lbo, unsigned int sbo)
    {
    return (unsigned long long)((addr >> 4) & 0x3fffu) | ((unsigned long long)((lbo >> 4) & 0x3fffu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
    }

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, both operands K-major, dense:
// D format (bits 4-5) = 1 (F32), A format (7-9) = 1 (BF16), B format (10-12) = 1 (BF16),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr unsigned int idesc_bf16_f32(unsigned int M, unsigned int N)
    {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
    }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned int count)
    {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned int parity)
    {
    unsigned int done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return done != 0u;
    }

// Waits for the phase of `parity` to complete, at most `limit` polls (each try_wait may suspend
// the thread for a short while); false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned int parity, unsigned int limit)
    {
    for (unsigned int i = 0; i < limit; ++i)
        {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 16u) __nanosleep(32);
        }
    return false;
    }

// Tensor Memory: `ncols` columns (a power of two >= 32) for this CTA, by one whole warp; the
// address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(unsigned int* dst, unsigned int ncols)
    {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

__device__ __forceinline__ void tmem_dealloc(unsigned int taddr, unsigned int ncols)
    {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
    }

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy stores to shared memory become visible to the tensor core's (async proxy) reads.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A[smem] x B[smem]^T, one thread issues.
__device__ __forceinline__ void mma_bf16(unsigned int d_tmem, unsigned long long a_desc, unsigned long long b_desc,
                                         unsigned int idesc, bool accumulate)
    {
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                 "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
                 : "memory");
    }

// The mbarrier receives one arrival when every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(unsigned long long* bar)
    {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
    }

// 16 consecutive 32-bit columns of this warp's 32 lanes (lane i of the warp gets TMEM lane
// base + i).  The registers are not valid until wait_ld() has run on them.
__device__ __forceinline__ void ld_32x32b_x16(unsigned int taddr, unsigned int (&r)[16])
    {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                 "[%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
    }

// Waits for this thread's outstanding tcgen05.ld; the registers pass through the statement, so
// that no use of them can be scheduled before the wait.  (Waiting again on registers of an earlier
// load costs nothing: the first wait covers every load issued before it.)
__device__ __forceinline__ void wait_ld(unsigned int (&r)[16])
    {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
    }

}  // namespace tc
}  // namespace gpu
}  // namespace neighbor

#endif
