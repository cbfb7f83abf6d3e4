// stage2.cu -- stage 2 of the step and the refresh of the stage-1 positions.
//
// One or TPR lanes per row of the padded position array.  For a real body they add the
// partial-sum slots of its segment (each lane its share, in slot order, then a fixed
// butterfly: deterministic), then lane 0 applies the base class's update in FP64 with
// separately rounded products and sums,
//     v = a*T + v ;  r = v*T + r          (_base_.py:58-62, np2.py:110-115)
// exactly as the reference's Python floats / numpy arrays round them, and finally
// rewrites the row of the stage-1 position array (FP32 hi[, lo] or FP64).  Padding
// rows get zeros (G*m = 0), so padded j-tiles contribute nothing.
#include "grav_device.cuh"

namespace grav {

struct __align__(32) drow4 {
	double x, y, z, w;
};

// Lanes per row: for small batches the row's slots are split over TPR adjacent lanes
// of a warp (lane p takes slots p, p + TPR, ...), so a few dozen slots cost one round
// of memory latency, and the lanes' partial sums are combined by a butterfly, which
// gives every lane the same bits.  For large batches one lane per row: there the extra
// lanes and their combining work cost more than the latency they hide.
constexpr int S2_THREADS = 128;
constexpr int SPLIT_ROWS_MAX = 32768;  // TPR = 4 up to this many padded rows, else 1
constexpr int ROW_BATCH = 8;           // FP64 row-slot loads in flight per lane
constexpr int COL_BATCH = 16;          // FP32 column-slot loads in flight per lane

// modes whose stage 1 reads the low parts of the positions (second float4 array)
__device__ __forceinline__ bool has_lo(int mode)
{
	return mode == GRAV_MODE_FP32C || mode == GRAV_MODE_FP32CU || mode == GRAV_MODE_FP32N ||
		mode == GRAV_MODE_FP32UN;
}

template <int TPR>
__global__ void __launch_bounds__(S2_THREADS) stage2_kernel(const grav_batch b, const int flags)
{
	static_assert(TPR > 0 && TPR <= 16 && (TPR & (TPR - 1)) == 0 && S2_THREADS % 32 == 0,
		"a row's lanes must sit in one warp");
	// launched as a dependent of stage 1; the next stage 1 may start launching when
	// this grid's CTAs exit (no earlier trigger: the persistent stage-1 grid should
	// find its SMs free)
	const int64_t gthread = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	const int64_t g = gthread / TPR;  // padded row; the TPR lanes of a row share a warp
	const int p = static_cast<int>(gthread % TPR);
	const unsigned gmask = ((1u << TPR) - 1) << ((threadIdx.x & 31) & ~(TPR - 1));
	if (g >= b.n_pad_total) return;  // the whole lane group
	const int IT = b.tile.bpt * b.tile.threads;
	const int64_t seg = g / IT;
	const int li = static_cast<int>(g - seg * IT);
	const grav_seg_desc S = b.seg[seg];
	const grav_univ_desc U = b.univ[S.u];
	const int il = S.il0 + li;
	// slots, positions and the state belong to the kernels before this one
	grid_dep_wait();

	if (il >= U.n) {  // the whole lane group
		if (p != 0) return;
		if (b.mode == GRAV_MODE_FP64) {
			static_cast<drow4*>(b.pos)[g] = drow4{0.0, 0.0, 0.0, 0.0};
		} else {
			float4* q = static_cast<float4*>(b.pos);
			q[g] = make_float4(0.f, 0.f, 0.f, 0.f);
			if (has_lo(b.mode)) q[b.n_pad_total + g] = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		return;
	}

	const int64_t row = U.body_off + il;
	drow4* rr = reinterpret_cast<drow4*>(b.r);
	drow4* vv = reinterpret_cast<drow4*>(b.v);
	const bool integrate = !(flags & GRAV_S2_PREPARE) && (flags & GRAV_S2_INTEGRATE);
	// lane 0 owns the row's update: its state loads go out before the slot loads
	drow4 r = {0.0, 0.0, 0.0, 0.0}, v = {0.0, 0.0, 0.0, 0.0};
	if (p == 0) {
		r = rr[row];
		if (integrate) v = vv[row];
	}

	double ax = 0.0, ay = 0.0, az = 0.0;
	if (!(flags & GRAV_S2_PREPARE)) {
		const int64_t stride = 3 * static_cast<int64_t>(IT);  // 8-byte entries per slot
		// unique-pair plans: the last (row block index) slots of a segment are column
		// slots holding FP32 sums in their first half (stage1_sym.cu)
		const bool pairs = b.mode == GRAV_MODE_FP32U || b.mode == GRAV_MODE_FP32CU ||
			b.mode == GRAV_MODE_FP32UN;
		const int nrow = pairs ? S.nslots - S.il0 / IT : S.nslots;
		if (b.mode == GRAV_MODE_FP64) {
			// FP64 row slots p, p + TPR, ... added in order; each round issues all its
			// loads first (the ones past the end are skipped): one latency per round
			const double* __restrict__ part =
				b.part + static_cast<int64_t>(S.slot_base) * stride + li;
			for (int k = p; k < nrow; k += ROW_BATCH * TPR) {
				const int m = min(ROW_BATCH, (nrow - k + TPR - 1) / TPR);
				double px[ROW_BATCH], py[ROW_BATCH], pz[ROW_BATCH];
#pragma unroll
				for (int q = 0; q < ROW_BATCH; ++q) {
					if (q < m) {
						const double* ps = part + (k + q * TPR) * stride;
						px[q] = __ldg(ps);
						py[q] = __ldg(ps + IT);
						pz[q] = __ldg(ps + 2 * IT);
					}
				}
#pragma unroll
				for (int q = 0; q < ROW_BATCH; ++q) {
					if (q < m) {
						ax += px[q];
						ay += py[q];
						az += pz[q];
					}
				}
			}
#pragma unroll
			for (int o = 1; o < TPR; o <<= 1) {
				ax += __shfl_xor_sync(gmask, ax, o);
				ay += __shfl_xor_sync(gmask, ay, o);
				az += __shfl_xor_sync(gmask, az, o);
			}
		} else {
			// FP32 modes: row slots hold the stage-1 pieces' compensated sums as FP32
			// (hi, lo) pairs; they and the column slots are added in slot order into a
			// compensated FP32 sum (hi by TwoSum, lo and the errors into L), combined
			// across the lanes by a TwoSum butterfly, and widened once.  No FP64
			// arithmetic per slot: GB300 runs FP64 at ~1/64 of the FP32 rate
			float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
			const float2* __restrict__ rpart =
				reinterpret_cast<const float2*>(b.part + static_cast<int64_t>(S.slot_base) * stride) + li;
			for (int k = p; k < nrow; k += ROW_BATCH * TPR) {
				const int m = min(ROW_BATCH, (nrow - k + TPR - 1) / TPR);
				float2 px[ROW_BATCH], py[ROW_BATCH], pz[ROW_BATCH];
#pragma unroll
				for (int q = 0; q < ROW_BATCH; ++q) {
					if (q < m) {
						const float2* ps = rpart + (k + q * TPR) * stride;
						px[q] = __ldg(ps);
						py[q] = __ldg(ps + IT);
						pz[q] = __ldg(ps + 2 * IT);
					}
				}
#pragma unroll
				for (int q = 0; q < ROW_BATCH; ++q) {
					if (q < m) {
						two_sum_acc(hx, lx, px[q].x);
						two_sum_acc(hy, ly, py[q].x);
						two_sum_acc(hz, lz, pz[q].x);
						lx += px[q].y;
						ly += py[q].y;
						lz += pz[q].y;
					}
				}
			}
			if (pairs) {
				// FP32 column slots; loads past the end read as 0, which TwoSum adds exactly
				const float* __restrict__ cpart = reinterpret_cast<const float*>(
					b.part + static_cast<int64_t>(S.slot_base) * stride) + li;
				const int64_t fstride = 2 * stride;  // floats per slot
				for (int k = nrow + p; k < S.nslots; k += COL_BATCH * TPR) {
					float px[COL_BATCH], py[COL_BATCH], pz[COL_BATCH];
#pragma unroll
					for (int q = 0; q < COL_BATCH; ++q) {
						px[q] = py[q] = pz[q] = 0.f;
						if (k + q * TPR < S.nslots) {
							const float* ps = cpart + (k + q * TPR) * fstride;
							px[q] = __ldg(ps);
							py[q] = __ldg(ps + IT);
							pz[q] = __ldg(ps + 2 * IT);
						}
					}
#pragma unroll
					for (int q = 0; q < COL_BATCH; ++q) {
						two_sum_acc(hx, lx, px[q]);
						two_sum_acc(hy, ly, py[q]);
						two_sum_acc(hz, lz, pz[q]);
					}
				}
			}
			group_sum_pair<TPR>(hx, lx, gmask);
			group_sum_pair<TPR>(hy, ly, gmask);
			group_sum_pair<TPR>(hz, lz, gmask);
			ax = static_cast<double>(hx) + static_cast<double>(lx);
			ay = static_cast<double>(hy) + static_cast<double>(ly);
			az = static_cast<double>(hz) + static_cast<double>(lz);
		}
	}
	if (p != 0) return;

	if (!(flags & GRAV_S2_PREPARE)) {
		if ((flags & GRAV_S2_WRITE_A) && b.a_out) {
			// streaming stores: a caller that keeps every step's accelerations writes a
			// new buffer each step, which must not push the step's own working set
			// (positions, slots, state) out of L2
			double2* ao = reinterpret_cast<double2*>(b.a_out) + 2 * row;
			__stcs(ao, make_double2(ax, ay));
			__stcs(ao + 1, make_double2(az, 0.0));
		}
		if (integrate) {
			const double T = U.T;
			v.x = __dadd_rn(__dmul_rn(ax, T), v.x);
			v.y = __dadd_rn(__dmul_rn(ay, T), v.y);
			v.z = __dadd_rn(__dmul_rn(az, T), v.z);
			r.x = __dadd_rn(__dmul_rn(v.x, T), r.x);
			r.y = __dadd_rn(__dmul_rn(v.y, T), r.y);
			r.z = __dadd_rn(__dmul_rn(v.z, T), r.z);
			vv[row] = v;
			rr[row] = r;
		}
	}

	if (b.mode == GRAV_MODE_FP64) {
		static_cast<drow4*>(b.pos)[g] = r;
	} else {
		float4* q = static_cast<float4*>(b.pos);
		const float hx = __double2float_rn(r.x);
		const float hy = __double2float_rn(r.y);
		const float hz = __double2float_rn(r.z);
		q[g] = make_float4(hx, hy, hz, __double2float_rn(r.w));
		if (has_lo(b.mode)) {
			q[b.n_pad_total + g] = make_float4(
				__double2float_rn(__dsub_rn(r.x, static_cast<double>(hx))),
				__double2float_rn(__dsub_rn(r.y, static_cast<double>(hy))),
				__double2float_rn(__dsub_rn(r.z, static_cast<double>(hz))), 0.f);
		}
	}
}

cudaError_t launch_stage2(const grav_batch& b, int flags, cudaStream_t stream, bool dependent)
{
	if (b.n_pad_total == 0) return cudaSuccess;
	const int tpr = b.n_pad_total <= SPLIT_ROWS_MAX ? 4 : 1;
	const int64_t blocks = (b.n_pad_total * tpr + S2_THREADS - 1) / S2_THREADS;
	grav_batch copy = b;
	int f = flags;
	void* args[] = {&copy, &f};
	const void* fn = tpr == 4 ? reinterpret_cast<const void*>(&stage2_kernel<4>)
	                          : reinterpret_cast<const void*>(&stage2_kernel<1>);
	if (!dependent)
		return cudaLaunchKernel(fn, dim3(static_cast<unsigned>(blocks)), dim3(S2_THREADS), args,
			0, stream);
	return launch_dependent(fn, static_cast<unsigned>(blocks), S2_THREADS, 0, stream, args);
}

}  // namespace grav
