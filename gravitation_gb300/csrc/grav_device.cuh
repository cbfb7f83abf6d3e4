// grav_device.cuh -- device-side helpers shared by the GB300 n-body kernels.
//
// Inline PTX for the SFU reciprocal square root, mbarrier waits with a time limit,
// and 1-D bulk (TMA) copies global -> shared.  Every spin-wait here is bounded:
// when the limit is reached the caller records an error code in device memory and
// returns, so that a lost copy never hangs the GPU.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "grav_types.h"

namespace grav {

// SFU reciprocal square root (MUFU), flush-to-zero.  For r2 > 0 normal inputs the
// result is within a few ulp of 1/sqrt(r2); the kernels guard r2 >= eps2 > 0.
__device__ __forceinline__ float rsqrt_sfu(float x)
{
	float y;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

// Make the initialised barriers visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
		"r"(bytes)
		: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(ok)
		: "r"(smem_addr(bar)), "r"(parity)
		: "memory");
	return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
	uint64_t t;
	asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
	return t;
}

// Bounded wait on one phase of an mbarrier.  Returns false when the phase has not
// completed after GRAV_WAIT_NS nanoseconds of polling (the clock is read every 16
// polls, so the bound holds whatever each poll's hardware suspend time is).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
	uint64_t limit_ns = GRAV_WAIT_NS)
{
	if (mbar_try_wait(bar, parity)) return true;
	const uint64_t t0 = global_ns();
	for (;;) {
		for (int k = 0; k < 16; ++k)
			if (mbar_try_wait(bar, parity)) return true;
		if (global_ns() - t0 > limit_ns) return false;
	}
}

// 1-D bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned) from
// global to this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes,
	uint64_t* bar)
{
	asm volatile(
		"cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
		::"r"(smem_addr(dst_smem)), "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
		: "memory");
}

// Compensated accumulation (Knuth's TwoSum, "The Art of Computer Programming" vol. 2,
// 4.2.2): hi + lo is the running sum; the rounding error of hi + x is kept exactly and
// added to lo.  Six FP32 additions; no FP64 (which runs at ~1/75 of the FP32 rate on
// this GPU).  Used to fold FP32 tile partials into a ~48-bit per-body sum.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x)
{
	const float s = hi + x;
	const float bp = s - hi;
	const float e = (hi - (s - bp)) + (x - bp);
	hi = s;
	lo += e;
}

// Record the first error code seen by any CTA.
__device__ __forceinline__ void set_error(int* err, int code)
{
	if (err) atomicCAS(err, 0, code);
}

}  // namespace grav
