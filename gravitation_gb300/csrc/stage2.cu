// stage2.cu -- stage 2 of the step and the refresh of the stage-1 positions.
//
// One thread per row of the padded position array.  For a real body it adds the
// FP64 partial-sum slots of its segment in slot order (deterministic), then applies
// the base class's update in FP64 with separately rounded products and sums,
//     v = a*T + v ;  r = v*T + r          (_base_.py:58-62, np2.py:110-115)
// exactly as the reference's Python floats / numpy arrays round them, and finally
// rewrites the row of the stage-1 position array (FP32 hi[, lo] or FP64).  Padding
// rows get zeros (G*m = 0), so padded j-tiles contribute nothing.
#include "grav_device.cuh"

namespace grav {

struct __align__(32) drow4 {
	double x, y, z, w;
};

__global__ void __launch_bounds__(256) stage2_kernel(const grav_batch b, const int flags)
{
	// launched as a dependent of stage 1; the next stage 1 may start launching when
	// this grid's CTAs exit (no earlier trigger: the persistent stage-1 grid should
	// find its SMs free)
	const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	if (g >= b.n_pad_total) return;
	const int IT = b.tile.bpt * b.tile.threads;
	const int64_t seg = g / IT;
	const int li = static_cast<int>(g - seg * IT);
	const grav_seg_desc S = b.seg[seg];
	const grav_univ_desc U = b.univ[S.u];
	const int il = S.il0 + li;
	// slots, positions and the state belong to the kernels before this one
	grid_dep_wait();

	if (il >= U.n) {
		if (b.mode == GRAV_MODE_FP64) {
			static_cast<drow4*>(b.pos)[g] = drow4{0.0, 0.0, 0.0, 0.0};
		} else {
			float4* p = static_cast<float4*>(b.pos);
			p[g] = make_float4(0.f, 0.f, 0.f, 0.f);
			if (b.mode == GRAV_MODE_FP32C || b.mode == GRAV_MODE_FP32CU)
				p[b.n_pad_total + g] = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		return;
	}

	const int64_t row = U.body_off + il;
	drow4* rr = reinterpret_cast<drow4*>(b.r);
	drow4 r = rr[row];

	if (!(flags & GRAV_S2_PREPARE)) {
		// slots are added in slot order; their loads are issued SLOT_BATCH at a time so
		// that a long slot list costs a few memory latencies, not one per slot
		constexpr int SLOT_BATCH = 8;
		double ax = 0.0, ay = 0.0, az = 0.0;
		const double* __restrict__ part = b.part + static_cast<int64_t>(S.slot_base) * 3 * IT + li;
		const int64_t stride = 3 * static_cast<int64_t>(IT);
		// unique-pair plans: the last (row block index) slots of a segment are column
		// slots holding FP32 sums in their first half (stage1_sym.cu)
		const bool pairs = b.mode == GRAV_MODE_FP32U || b.mode == GRAV_MODE_FP32CU;
		const int nrow = pairs ? S.nslots - S.il0 / IT : S.nslots;
		int k = 0;
		for (; k + SLOT_BATCH <= nrow; k += SLOT_BATCH) {
			double px[SLOT_BATCH], py[SLOT_BATCH], pz[SLOT_BATCH];
#pragma unroll
			for (int q = 0; q < SLOT_BATCH; ++q) {
				const double* p = part + (k + q) * stride;
				px[q] = __ldg(p);
				py[q] = __ldg(p + IT);
				pz[q] = __ldg(p + 2 * IT);
			}
#pragma unroll
			for (int q = 0; q < SLOT_BATCH; ++q) {
				ax += px[q];
				ay += py[q];
				az += pz[q];
			}
		}
		for (; k < nrow; ++k) {
			const double* p = part + k * stride;
			ax += __ldg(p);
			ay += __ldg(p + IT);
			az += __ldg(p + 2 * IT);
		}
		// column slots: FP32 values added in slot order by TwoSum in FP32 (hi + lo,
		// ~48 bits) and widened once.  With FP64 adds and conversions per slot (64
		// column slots per row at N = 65536) the FP64 pipe, ~1/64 of the FP32 rate on
		// GB300, bound this kernel
		const float* __restrict__ cpart =
			reinterpret_cast<const float*>(b.part + static_cast<int64_t>(S.slot_base) * 3 * IT) + li;
		const int64_t fstride = 2 * stride;  // floats per slot
		float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
		for (; k + SLOT_BATCH <= S.nslots; k += SLOT_BATCH) {
			float px[SLOT_BATCH], py[SLOT_BATCH], pz[SLOT_BATCH];
#pragma unroll
			for (int q = 0; q < SLOT_BATCH; ++q) {
				const float* p = cpart + (k + q) * fstride;
				px[q] = __ldg(p);
				py[q] = __ldg(p + IT);
				pz[q] = __ldg(p + 2 * IT);
			}
#pragma unroll
			for (int q = 0; q < SLOT_BATCH; ++q) {
				two_sum_acc(hx, lx, px[q]);
				two_sum_acc(hy, ly, py[q]);
				two_sum_acc(hz, lz, pz[q]);
			}
		}
		for (; k < S.nslots; ++k) {
			const float* p = cpart + k * fstride;
			two_sum_acc(hx, lx, __ldg(p));
			two_sum_acc(hy, ly, __ldg(p + IT));
			two_sum_acc(hz, lz, __ldg(p + 2 * IT));
		}
		ax += static_cast<double>(hx) + static_cast<double>(lx);
		ay += static_cast<double>(hy) + static_cast<double>(ly);
		az += static_cast<double>(hz) + static_cast<double>(lz);
		if ((flags & GRAV_S2_WRITE_A) && b.a_out)
			reinterpret_cast<drow4*>(b.a_out)[row] = drow4{ax, ay, az, 0.0};
		if (flags & GRAV_S2_INTEGRATE) {
			drow4* vv = reinterpret_cast<drow4*>(b.v);
			drow4 v = vv[row];
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
		float4* p = static_cast<float4*>(b.pos);
		const float hx = __double2float_rn(r.x);
		const float hy = __double2float_rn(r.y);
		const float hz = __double2float_rn(r.z);
		p[g] = make_float4(hx, hy, hz, __double2float_rn(r.w));
		if (b.mode == GRAV_MODE_FP32C || b.mode == GRAV_MODE_FP32CU) {
			p[b.n_pad_total + g] = make_float4(
				__double2float_rn(__dsub_rn(r.x, static_cast<double>(hx))),
				__double2float_rn(__dsub_rn(r.y, static_cast<double>(hy))),
				__double2float_rn(__dsub_rn(r.z, static_cast<double>(hz))), 0.f);
		}
	}
}

cudaError_t launch_stage2(const grav_batch& b, int flags, cudaStream_t stream)
{
	if (b.n_pad_total == 0) return cudaSuccess;
	// small CTAs: a few thousand rows still spread over many SMs (latency bound)
	const int threads = 64;
	const int64_t blocks = (b.n_pad_total + threads - 1) / threads;
	grav_batch copy = b;
	int f = flags;
	void* args[] = {&copy, &f};
	return launch_dependent(reinterpret_cast<const void*>(&stage2_kernel),
		static_cast<unsigned>(blocks), threads, 0, stream, args);
}

}  // namespace grav
