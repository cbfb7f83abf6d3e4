// stage1_f64.cu -- stage 1 (all-pairs accelerations) in GRAV_MODE_FP64.
//
// Same persistent stream-K decomposition and bulk-copy pipeline as stage1_f32.cu,
// with FP64 positions (x, y, z, G*m) in the tiles and FP64 arithmetic throughout:
//     d = r_j - r_i ;  r2 = |d|^2 ;  w = Gm_j / r2^(3/2) (0 when r2 == 0) ;  a += w d
// which is the reference's law (np1.py:81-95, py1.py:57-64) in double precision.
// The GB300 runs FP64 at a small fraction of its FP32 rate, so this mode is the
// accuracy reference on the GPU, not the fast path.
#include "grav_device.cuh"

namespace grav {

struct __align__(32) dpos4 {
	double x, y, z, w;
};

template <int B, int T, int J>
__global__ void __launch_bounds__(T) stage1_f64_kernel(const grav_batch b)
{
	constexpr int IT = B * T;
	constexpr uint32_t TILE_BYTES = J * sizeof(dpos4);
	extern __shared__ __align__(128) dpos4 smem_dtiles[];  // [2][J]
	__shared__ __align__(8) uint64_t bar[2];

	const int tid = threadIdx.x;
	const int64_t U = b.n_units;
	const int64_t G = gridDim.x;
	const int64_t c = blockIdx.x;
	int64_t ub = c * U / G;
	const int64_t ue = (c + 1) * U / G;
	if (ub >= ue) return;

	if (tid == 0) {
		mbar_init(&bar[0], 1);
		mbar_init(&bar[1], 1);
		fence_barrier_init();
	}
	__syncthreads();

	const dpos4* __restrict__ pos = static_cast<const dpos4*>(b.pos);

	int s = find_segment(b.seg, b.n_seg, ub);
	// positions and partial-sum slots belong to the kernels before this one
	grid_dep_wait();

	uint32_t gt = 0;
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
		const dpos4* __restrict__ jsrc = pos + Uu.pad_off;

		if (tid == 0) {
			const int bs = gt & 1;
			mbar_arrive_expect_tx(&bar[bs], TILE_BYTES);
			bulk_g2s(smem_dtiles + bs * J, jsrc + jt0 * J, TILE_BYTES, &bar[bs]);
		}

		double xi[B], yi[B], zi[B], ax[B], ay[B], az[B];
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const dpos4 p = pos[ibase + tid + k * T];
			xi[k] = p.x;
			yi[k] = p.y;
			zi[k] = p.z;
			ax[k] = ay[k] = az[k] = 0.0;
		}

		for (int t = 0; t < nt; ++t, ++gt) {
			const int bs = gt & 1;
			const bool ok = mbar_wait_bounded(&bar[bs], (gt >> 1) & 1);
			if (__syncthreads_or(!ok)) {
				timed_out = true;
				break;
			}
			if (tid == 0 && t + 1 < nt) {
				const int bn = (gt + 1) & 1;
				mbar_arrive_expect_tx(&bar[bn], TILE_BYTES);
				bulk_g2s(smem_dtiles + bn * J, jsrc + (jt0 + t + 1) * J, TILE_BYTES, &bar[bn]);
			}
			const dpos4* __restrict__ sj = smem_dtiles + bs * J;
#pragma unroll 2
			for (int j = 0; j < J; ++j) {
				const dpos4 pj = sj[j];
#pragma unroll
				for (int k = 0; k < B; ++k) {
					const double dx = pj.x - xi[k];
					const double dy = pj.y - yi[k];
					const double dz = pj.z - zi[k];
					const double r2 = dx * dx + dy * dy + dz * dz;
					const double inv = (r2 > 0.0) ? rsqrt(r2) : 0.0;
					const double w = pj.w * (inv * inv * inv);
					ax[k] += w * dx;
					ay[k] += w * dy;
					az[k] += w * dz;
				}
			}
		}
		if (timed_out) break;

		const int64_t slot = S.slot_base + (c - S.cta_first);
		double* __restrict__ out = b.part + slot * 3 * IT;
#pragma unroll
		for (int k = 0; k < B; ++k) {
			out[tid + k * T] = ax[k];
			out[IT + tid + k * T] = ay[k];
			out[2 * IT + tid + k * T] = az[k];
		}
		ub = S.unit_begin + jt1;
		++s;
	}

	// the next kernel in the stream may start launching now (it waits for this grid)
	grid_dep_launch();
	if (timed_out && tid == 0) {
		set_error(b.err, GRAV_DEV_TIMEOUT);
		mbar_wait_bounded(&bar[gt & 1], (gt >> 1) & 1);
	}
}

#define GRAV_F64_ENTRY(B, T, J) \
	{GRAV_MODE_FP64, B, T, J, reinterpret_cast<const void*>(&stage1_f64_kernel<B, T, J>), \
		2 * J * 32, true}

static const Stage1Kernel k_table_f64[] = {
	GRAV_F64_ENTRY(1, 128, 128),
	GRAV_F64_ENTRY(2, 128, 128),
	GRAV_F64_ENTRY(1, 256, 128),
	GRAV_F64_ENTRY(2, 256, 128),
};

int stage1_table_f64(const Stage1Kernel** out)
{
	*out = k_table_f64;
	return static_cast<int>(sizeof(k_table_f64) / sizeof(k_table_f64[0]));
}

}  // namespace grav
