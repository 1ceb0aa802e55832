/*
 * Fifth-generation tensor-core primitives (tcgen05) for BF16 GEMM tiles:
 * tensor-memory allocation, shared-memory matrix descriptors in the
 * no-swizzle K-major layout, the single-thread MMA issue with its commit to
 * an mbarrier, and tensor-memory loads of the FP32 accumulator.
 *
 * Operand layout in shared memory (no swizzle, K-major): core matrices of
 * 8 rows x 16 bytes (8 BF16 of K), 128 contiguous bytes each; element (m, k)
 * of an operand with R rows sits at byte (k / 8) * LBO + m * 16 + (k % 8) * 2
 * with LBO = 16 R, i.e. the 8-row groups of a K-chunk are adjacent (SBO = 128
 * bytes) and the K-chunks follow one another.  One MMA instruction consumes
 * K = 16: two K-chunks, LBO apart.
 */
#pragma once

#include <cstdint>

namespace fvg {

/* instruction descriptor of tcgen05.mma kind::f16: D FP32, A and B BF16,
 * both K-major, shape M x N */
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N)
{
	return (1u << 4)                      // D format: FP32
	       | (1u << 7)                    // A format: BF16
	       | (1u << 10)                   // B format: BF16
	       | ((uint32_t)(N >> 3) << 17)   // N / 8
	       | ((uint32_t)(M >> 4) << 24);  // M / 16
}

/* shared-memory descriptor, no swizzle: start address, leading (K-chunk)
 * byte offset, stride (8-row group) byte offset */
__device__ __forceinline__ uint64_t tc_sdesc(unsigned saddr, unsigned lbo, unsigned sbo)
{
	return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
	       ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* warp-wide: allocates ncols (a power of two >= 32) tensor-memory columns;
 * the address lands in *slot (shared memory) */
__device__ __forceinline__ void tc_alloc(uint32_t *slot, unsigned ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(slot)),
	             "r"(ncols)
	             : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

/* warp-wide: frees the columns of tc_alloc */
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, unsigned ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

/* one thread: D (+)= A B^T for one K = 16 step */
__device__ __forceinline__ void tc_mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            int accumulate)
{
	asm volatile(
	    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
	    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
	    : "memory");
}

/* one thread: the mbarrier receives one arrival when this thread's issued
 * MMAs have completed */
__device__ __forceinline__ void tc_commit(uint64_t *bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
	                 smem_u32(bar))
	             : "memory");
}

/* warp-wide: 16 consecutive FP32 columns of the warp's 32 tensor-memory lanes
 * (thread i: lane base + i) */
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float *v)
{
	uint32_t r[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr)
	    : "memory");
	// the wait names the loaded registers, so no use of them moves above it
	asm volatile("tcgen05.wait::ld.sync.aligned;\n"
	             : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
	               "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
	             :
	             : "memory");
#pragma unroll
	for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

}  // namespace fvg
