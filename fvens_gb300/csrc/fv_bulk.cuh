/*
 * Bulk asynchronous copies (the TMA engine's untiled form,
 * cp.async.bulk.shared::cluster.global) from global into shared memory, with
 * completion counted on a shared-memory mbarrier (complete_tx), and a wait
 * bounded in time: a wait that runs out returns false, and the caller records
 * an error and ends its CTA once its copies have landed.
 *
 * Alignment: both addresses 16-byte aligned and the size a multiple of 16.
 */
#pragma once

#include <cstdint>

namespace fvg {

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}

/* the initialised barriers become visible to the async proxy (bulk copies) */
__device__ __forceinline__ void mbar_init_fence()
{
	asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

/* orders this thread's earlier generic-proxy accesses of shared memory before
 * later async-proxy writes (a buffer read by the CTA is refilled by a copy) */
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

/* one arrival that also expects `bytes` of transactions on the barrier */
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
	             : "memory");
}

/* global -> shared bulk copy of `bytes`, counted on bar */
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
	asm volatile(
	    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
	        smem_u32(dst)),
	    "l"(src), "r"(bytes), "r"(smem_u32(bar))
	    : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
	unsigned ok;
	asm volatile(
	    "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
	    : "=r"(ok)
	    : "r"(smem_u32(bar)), "r"(parity)
	    : "memory");
	return ok != 0;
}

/* waits for the phase with the given parity to complete; false after about
 * `limit_cycles` SM clocks without completion */
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, long long limit_cycles = 2000000000LL)
{
	const long long t0 = clock64();
	while (!mbar_try_wait(bar, parity))
		if (clock64() - t0 > limit_cycles) return false;
	return true;
}

}  // namespace fvg
