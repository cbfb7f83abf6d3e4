// stage1_f32.cu -- stage 1 (all-pairs accelerations) in the FP32 precision modes.
//
// Force law of the reference (np1.py:81-95, py1.py:57-64, pc2.py:75-89):
//     a_i = sum_{j != i} G m_j (r_j - r_i) / |r_j - r_i|^3
// evaluated as   d = r_j - r_i ;  r2 = |d|^2 + eps2 ;  w = Gm_j * rsqrt(r2)^3 ;  a += w d
// with 12 FMA-pipe operations and one SFU reciprocal square root per interaction.
// eps2 (grav_eps2) only keeps the zero-separation terms finite so that they vanish
// with d = 0; it is absorbed by rounding for any separation the FP32 coordinates
// resolve, so it is not a softening length.
//
// Work decomposition (persistent, "stream-K" over j-tiles): the plan lists every
// (universe, i-tile) segment; each segment owns one work unit per j-tile of its
// universe.  CTA c of G processes the contiguous unit range [c*U/G, (c+1)*U/G), so
// every CTA gets the same number of j-tiles (+-1) whatever the universe sizes are.
// Per segment a CTA holds B i-bodies per thread in registers, streams its j-tiles
// through double-buffered shared memory with 1-D bulk copies (cp.async.bulk,
// completion on an mbarrier), sums each j-tile's contribution in FP32 and folds
// that partial into a compensated FP32 sum (TwoSum hi + lo, ~48 bits, no FP64 in the
// loop).  The CTA's piece of the segment goes as FP64 to its own slot of b.part;
// stage 2 adds the slots in FP64 in a fixed order, so results do not depend on
// scheduling.
//
// GRAV_MODE_FP32C reads a second FP32 array with the low parts of the positions
// (x = hi + lo) and forms d = (hi_j - hi_i) + (lo_j - lo_i): the separation is then
// accurate to FP32 relative precision however far the bodies are from the origin.
// GRAV_MODE_FP32N keeps the FP32 loop and compares each pair's r2 with the near radius
// (grav_device.cuh, near_threshold); a step where any lane of the warp met a nearer
// pair re-evaluates those pairs from the double-single separation (near_delta).  The
// j-tiles that hold the CTA's own rows also require r2 > eps2, so that the self pairs
// (d = 0) do not send every warp down that cold path.
#include "grav_device.cuh"

namespace grav {

template <int MODE, int B, int T, int J>
__global__ void __launch_bounds__(T) stage1_f32_kernel(const grav_batch b)
{
	constexpr bool DS = MODE == GRAV_MODE_FP32C;            // double-single separations
	constexpr bool NEAR = MODE == GRAV_MODE_FP32N;          // ... for near pairs only
	constexpr int NP = (DS || NEAR) ? 2 : 1;                // float4 arrays per body
	constexpr int IT = B * T;                               // i-tile
	constexpr uint32_t TILE_BYTES = J * sizeof(float4);
	extern __shared__ __align__(128) float4 smem_tiles[];   // [2 buffers][NP][J]
	__shared__ __align__(8) uint64_t bar[2];
	// low parts of this thread's rows (NEAR), read back only by the thread that wrote them
	__shared__ float4 rowlo[NEAR ? B : 1][NEAR ? T : 1];

	const int tid = threadIdx.x;
	const int64_t U = b.n_units;
	const int64_t G = gridDim.x;
	const int64_t c = blockIdx.x;
	int64_t ub = c * U / G;
	const int64_t ue = (c + 1) * U / G;
	if (ub >= ue) return;  // uniform over the CTA

	if (tid == 0) {
		mbar_init(&bar[0], 1);
		mbar_init(&bar[1], 1);
		fence_barrier_init();
	}
	__syncthreads();

	const float4* __restrict__ pos = static_cast<const float4*>(b.pos);
	const float4* __restrict__ poslo = pos + b.n_pad_total;
	const float eps2 = b.eps2;

	// segment holding unit ub: the last segment whose unit_begin <= ub
	int s = find_segment(b.seg, b.n_seg, ub);
	// positions and partial-sum slots belong to the kernels before this one
	grid_dep_wait();

	uint32_t gt = 0;  // tiles consumed by this CTA so far (buffer gt&1, parity (gt>>1)&1)
	bool timed_out = false;

	while (ub < ue && s < b.n_seg) {
		const grav_seg_desc S = b.seg[s];
		if (S.n_units == 0 || S.unit_begin + S.n_units <= ub) {
			++s;
			continue;
		}
		const grav_univ_desc Uu = b.univ[S.u];
		const int64_t jt0 = ub - S.unit_begin;
		const int64_t jt1 = min(ue - S.unit_begin, (int64_t)S.n_units);
		const int nt = static_cast<int>(jt1 - jt0);
		const int64_t ibase = Uu.pad_off + S.il0;
		const float4* __restrict__ jsrc = pos + Uu.pad_off;
		const float4* __restrict__ jsrclo = poslo + Uu.pad_off;

		// first j-tile of this piece; buffer gt&1 was last read two tiles ago and every
		// thread has passed a barrier since
		if (tid == 0) {
			const int bs = gt & 1;
			mbar_arrive_expect_tx(&bar[bs], NP * TILE_BYTES);
			bulk_g2s(smem_tiles + (bs * NP) * J, jsrc + jt0 * J, TILE_BYTES, &bar[bs]);
			if (NP == 2)
				bulk_g2s(smem_tiles + (bs * NP + 1) * J, jsrclo + jt0 * J, TILE_BYTES, &bar[bs]);
		}

		float xi[B], yi[B], zi[B];
		float xl[B], yl[B], zl[B];
		float fx[B], fy[B], fz[B];
		float hx[B], hy[B], hz[B], lx[B], ly[B], lz[B];  // compensated per-body sums
		float xmax = 0.f;                                // NEAR: largest |coordinate| of the rows
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const float4 p = pos[ibase + tid + k * T];
			xi[k] = p.x;
			yi[k] = p.y;
			zi[k] = p.z;
			if (DS) {
				const float4 q = poslo[ibase + tid + k * T];
				xl[k] = q.x;
				yl[k] = q.y;
				zl[k] = q.z;
			} else {
				xl[k] = yl[k] = zl[k] = 0.f;
			}
			if (NEAR) {
				rowlo[NEAR ? k : 0][NEAR ? tid : 0] = poslo[ibase + tid + k * T];
				xmax = fmaxf(xmax, near_scale(p.x, p.y, p.z));
			}
			fx[k] = fy[k] = fz[k] = 0.f;
			hx[k] = hy[k] = hz[k] = lx[k] = ly[k] = lz[k] = 0.f;
		}
		const float thr = near_threshold(xmax);

		for (int t = 0; t < nt; ++t, ++gt) {
			const int bs = gt & 1;
			const bool ok = mbar_wait_bounded(&bar[bs], (gt >> 1) & 1);
			if (__syncthreads_or(!ok)) {
				timed_out = true;
				break;
			}
			if (tid == 0 && t + 1 < nt) {
				const int bn = (gt + 1) & 1;
				const int64_t jt = jt0 + t + 1;
				mbar_arrive_expect_tx(&bar[bn], NP * TILE_BYTES);
				bulk_g2s(smem_tiles + (bn * NP) * J, jsrc + jt * J, TILE_BYTES, &bar[bn]);
				if (NP == 2)
					bulk_g2s(smem_tiles + (bn * NP + 1) * J, jsrclo + jt * J, TILE_BYTES, &bar[bn]);
			}
			const float4* __restrict__ sj = smem_tiles + (bs * NP) * J;
			const float4* __restrict__ sl = sj + J;
			// NEAR: does this j-tile hold rows of this CTA (their self pairs)?
			const int64_t jl0 = (jt0 + t) * J;
			const bool own = jl0 < S.il0 + IT && jl0 + J > S.il0;
			if (NEAR && own)
				rows_tile<B, J, DS, NEAR, true>(sj, sl, eps2, thr, xi, yi, zi, xl, yl, zl, fx, fy,
					fz, &rowlo[0][0], tid, T);
			else
				rows_tile<B, J, DS, NEAR, false>(sj, sl, eps2, thr, xi, yi, zi, xl, yl, zl, fx, fy,
					fz, &rowlo[0][0], tid, T);
#pragma unroll
			for (int k = 0; k < B; ++k) {
				two_sum_acc(hx[k], lx[k], fx[k]);
				two_sum_acc(hy[k], ly[k], fy[k]);
				two_sum_acc(hz[k], lz[k], fz[k]);
				fx[k] = fy[k] = fz[k] = 0.f;
			}
		}
		if (timed_out) break;

		// this CTA's piece of the segment: the compensated sums go out as FP32 (hi, lo)
		// pairs, one 8-byte slot entry each, with no FP64 arithmetic (GB300 runs FP64 at
		// ~1/64 of the FP32 rate); stage 2 adds the pairs in FP32 by TwoSum
		const int64_t slot = S.slot_base + (c - S.cta_first);
		float2* __restrict__ out = reinterpret_cast<float2*>(b.part + slot * 3 * IT);
#pragma unroll
		for (int k = 0; k < B; ++k) {
			out[tid + k * T] = make_float2(hx[k], lx[k]);
			out[IT + tid + k * T] = make_float2(hy[k], ly[k]);
			out[2 * IT + tid + k * T] = make_float2(hz[k], lz[k]);
		}
		ub = S.unit_begin + jt1;
		++s;
	}

	// the next kernel in the stream may start launching now (it waits for this grid);
	// not earlier, so that its CTAs find the SMs this persistent grid leaves
	grid_dep_launch();
	if (timed_out && tid == 0) {
		set_error(b.err, GRAV_DEV_TIMEOUT);
		// the copy that did not arrive is the only one in flight; give it one more
		// bounded wait so that it does not land in shared memory after this CTA exits
		mbar_wait_bounded(&bar[gt & 1], (gt >> 1) & 1);
	}
}

#define GRAV_F32_ENTRY(MODE, B, T, J) \
	{MODE, B, T, J, reinterpret_cast<const void*>(&stage1_f32_kernel<MODE, B, T, J>), \
		2 * ((MODE == GRAV_MODE_FP32) ? 1 : 2) * J * 16, true}

static const Stage1Kernel k_table_f32[] = {
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 1, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 2, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 4, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 4, 128, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 8, 128, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 2, 256, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 4, 256, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32, 8, 256, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32C, 1, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32C, 2, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32C, 4, 128, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32C, 4, 256, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32N, 1, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32N, 2, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32N, 4, 128, 128),
	GRAV_F32_ENTRY(GRAV_MODE_FP32N, 4, 128, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32N, 8, 128, 256),
	GRAV_F32_ENTRY(GRAV_MODE_FP32N, 4, 256, 256),
};

int stage1_table_f32(const Stage1Kernel** out)
{
	*out = k_table_f32;
	return static_cast<int>(sizeof(k_table_f32) / sizeof(k_table_f32[0]));
}

}  // namespace grav
