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

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while the kernel before it in the stream is still running:
// grid_dep_wait() blocks until that kernel has completed and its memory operations are
// visible, so everything before it may only read data no earlier kernel writes (plan
// tables, launch arguments).  grid_dep_launch() lets the next kernel in the stream
// start its own launch.  Both are no-ops for a kernel launched the ordinary way.
__device__ __forceinline__ void grid_dep_wait()
{
	asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void grid_dep_launch()
{
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Near-pair correction (GRAV_MODE_FP32N / GRAV_MODE_FP32UN).  Rounding a coordinate x
// to FP32 moves it by up to 2^-24 |x|, so the FP32 separation of two bodies far from the
// origin but close to each other carries a relative error of order 2^-24 |x| / |d|.
// The near modes evaluate every pair with r2 < near_threshold() (|d| below
// max|x| / GRAV_NEAR_KAPPA, max|x| over the coordinates of the thread's rows) a second
// time from the double-single separation d_a = (hi_j - hi_i) + (lo_j - lo_i) and add the
// difference.  Beyond that distance the FP32 separation is within
// 2^-24 (sqrt(3) (2 kappa + 1) + 1) of the exact one (~4.5e-6 relative pair-force error
// at kappa = 20, a bound; measured body errors stay below 1e-6).
__device__ __forceinline__ float near_scale(float x, float y, float z)
{
	return fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z)));
}

__device__ __forceinline__ float near_threshold(float max_abs_coord)
{
	constexpr float inv_k2 = 1.0f / (GRAV_NEAR_KAPPA * GRAV_NEAR_KAPPA);
	return max_abs_coord * max_abs_coord * inv_k2;
}

// Running minimum of the r2 values of a thread's B rows for the near test, one
// three-input min per two rows (min.f32 with three operands, sm_100 and later): call
// with k = 0 .. B-1 in order; `prev` holds the previous row's r2 between calls.
__device__ __forceinline__ float min3f(float a, float b, float c)
{
	float r;
	asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
	return r;
}

template <int B>
__device__ __forceinline__ void near_min_step(int k, float r2, float& m, float& prev)
{
	if (k == 0) m = r2;
	else if ((k & 1) == 0) m = min3f(m, prev, r2);
	else if (k == B - 1) m = fminf(m, r2);
	prev = r2;
}

// (ex, ey, ez) = d_a |d_a|^-3 - d |d|^-3 for the pair whose FP32 separation is (dx, dy,
// dz) with r2 = |d|^2 + eps2 (as the main loop formed it), lj / li the low parts of the
// column and row bodies; zero unless `on`.  The caller adds Gm_j e to the row's sum and
// -Gm_i e to the column's, which replaces the FP32 pair term by the double-single one.
__device__ __forceinline__ void near_delta(float dx, float dy, float dz, float r2,
	const float4& lj, const float4& li, float eps2, bool on, float& ex, float& ey, float& ez)
{
	const float ax = dx + (lj.x - li.x);
	const float ay = dy + (lj.y - li.y);
	const float az = dz + (lj.z - li.z);
	const float ra2 = fmaf(az, az, fmaf(ay, ay, fmaf(ax, ax, eps2)));
	const float ia = rsqrt_sfu(ra2);
	const float ia3 = ia * (ia * ia);
	const float i1 = rsqrt_sfu(r2);
	const float i3 = i1 * (i1 * i1);
	ex = on ? fmaf(ax, ia3, -(dx * i3)) : 0.f;
	ey = on ? fmaf(ay, ia3, -(dy * i3)) : 0.f;
	ez = on ? fmaf(az, ia3, -(dz * i3)) : 0.f;
}

// One j-tile against a thread's B rows, every ordered pair, rows only: the inner loop
// of the all-pairs kernel (stage1_f32.cu); the rows' low parts are rowlo[k * T + tid].
// (The unique-pair kernel keeps its own copy of this loop with a test per step: with
// this function inlined there its main loop compiled measurably slower on GB300.)  NEAR adds the near
// test (one three-input min per two rows and a compare; with SELF -- tiles that hold the
// thread block's own rows -- a test per pair that also excludes r2 = eps2, so that self
// pairs do not count) whose result is a bit per step, and after every 32 steps a cold
// path over the steps where some lane of the warp met a near pair.
template <int B, int JT, bool DS, bool NEAR, bool SELF>
__device__ __forceinline__ void rows_tile(const float4* __restrict__ sj,
	const float4* __restrict__ sjl, float eps2, float thr, const float (&xi)[B],
	const float (&yi)[B], const float (&zi)[B], const float (&xl)[B], const float (&yl)[B],
	const float (&zl)[B], float (&fx)[B], float (&fy)[B], float (&fz)[B],
	const float4* __restrict__ rowlo, int tid, int T)
{
	static_assert(JT % 32 == 0, "j-tiles of whole 32-body groups");
#pragma unroll 1
	for (int j0 = 0; j0 < JT; j0 += 32) {
		uint32_t nmask = 0;
#pragma unroll 4
		for (int jj = 0; jj < 32; ++jj) {
			const float4 pj = sj[j0 + jj];
			float4 lj = make_float4(0.f, 0.f, 0.f, 0.f);
			if (DS) lj = sjl[j0 + jj];
			float rmin = 0.f, rprev = 0.f;
			bool near = false;
#pragma unroll
			for (int k = 0; k < B; ++k) {
				float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
				if (DS) {
					dx = dx + (lj.x - xl[k]);
					dy = dy + (lj.y - yl[k]);
					dz = dz + (lj.z - zl[k]);
				}
				const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
				if (NEAR && SELF) near |= (r2 < thr) & (r2 > eps2);
				if (NEAR && !SELF) near_min_step<B>(k, r2, rmin, rprev);
				const float inv = rsqrt_sfu(r2);
				float w = pj.w * inv;
				w = w * (inv * inv);
				fx[k] = fmaf(dx, w, fx[k]);
				fy[k] = fmaf(dy, w, fy[k]);
				fz[k] = fmaf(dz, w, fz[k]);
			}
			if (NEAR && !SELF) near = rmin < thr;
			if (NEAR && near) nmask |= 1u << jj;
		}
		if (NEAR) {
			uint32_t todo = __reduce_or_sync(0xffffffffu, nmask);
			while (todo) {
				const int jj = __ffs(todo) - 1;
				todo &= todo - 1;
				const float4 pj = sj[j0 + jj];
				const float4 lj = sjl[j0 + jj];
#pragma unroll
				for (int k = 0; k < B; ++k) {
					const float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
					const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
					const bool nk = (r2 < thr) & (r2 > eps2);
					if (__any_sync(0xffffffffu, nk)) {
						float ex, ey, ez;
						near_delta(dx, dy, dz, r2, lj, rowlo[k * T + tid], eps2, nk, ex, ey, ez);
						fx[k] = fmaf(ex, pj.w, fx[k]);
						fy[k] = fmaf(ey, pj.w, fy[k]);
						fz[k] = fmaf(ez, pj.w, fz[k]);
					}
				}
			}
		}
	}
}

// Combine the compensated FP32 sums (H, L) of the WIDTH lanes of an aligned lane group
// by an xor butterfly: H by TwoSum, L and the rounding error added.  Every lane ends
// with the same bits: TwoSum's error term is the exact rounding error of H_a + H_b in
// either operand order, and FP32 addition commutes.
template <int WIDTH>
__device__ __forceinline__ void group_sum_pair(float& H, float& L, unsigned mask)
{
#pragma unroll
	for (int o = 1; o < WIDTH; o <<= 1) {
		const float hb = __shfl_xor_sync(mask, H, o);
		const float lb = __shfl_xor_sync(mask, L, o);
		const float s = H + hb;
		const float bp = s - H;
		const float e = (H - (s - bp)) + (hb - bp);
		H = s;
		L = (L + lb) + e;
	}
}

// Record the first error code seen by any CTA.
__device__ __forceinline__ void set_error(int* err, int code)
{
	if (err) atomicCAS(err, 0, code);
}

// Index of the last plan segment whose unit_begin <= ub (unit_begin never decreases
// along the table and seg[0].unit_begin = 0 <= ub).  Each warp searches on its own:
// per round its 32 lanes probe 32 evenly spaced candidates and a ballot keeps the
// interval between the last candidate that qualifies and the next one, so the search
// takes ceil(log32(n_seg)) rounds of independent loads where a bisection takes
// log2(n_seg) dependent ones.  All 32 lanes of the warp must call it together.
__device__ __forceinline__ int find_segment(const grav_seg_desc* seg, int n_seg, int64_t ub)
{
	const unsigned full = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	int lo = 0, hi = n_seg - 1;
	while (lo < hi) {
		const int span = hi - lo + 1;  // candidates left, >= 2
		const int idx = span <= 32 ? lo + min(lane, span - 1)
		                           : lo + static_cast<int>((static_cast<int64_t>(lane) * span) / 32);
		const unsigned ok = __ballot_sync(full, seg[idx].unit_begin <= ub);  // lane 0 qualifies
		const int top = 31 - __clz(ok);
		const int at = __shfl_sync(full, idx, top);
		const int after = __shfl_sync(full, idx, (top + 1) & 31);
		if (span <= 32) return at;
		hi = top < 31 ? after - 1 : hi;
		lo = at;
	}
	return lo;
}

}  // namespace grav
