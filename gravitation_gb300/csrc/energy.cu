// energy.cu -- FP64 energy and momentum of every universe of a batch.
//
// The reference has no energy diagnostic (an "accuracy" command is a wish, TODO.md:4);
// the precision modes are compared by the drift of
//     E = sum_i 1/2 m_i v_i^2  -  sum_{i<j} G m_i m_j / |r_i - r_j|      and   P = sum_i m_i v_i
// over a run.  Both are computed in FP64 from the FP64 state with G*m in r[:,3]:
//   pass 1 (persistent, the stage-1 work list): phi_i = sum_{j!=i} Gm_j / |r_j - r_i|
//          into the partial-sum slots (one value per body and slot)
//   pass 2 (one CTA per universe): K = sum 1/2 Gm v^2, W = -1/2 sum Gm_i phi_i,
//          P = sum Gm v, reduced in a fixed order; dividing by G gives energy/momentum.
#include "pairs_skeleton.cuh"

namespace grav {

struct __align__(32) epos4 {
	double x, y, z, w;
};

template <int B_, int T_, int J_>
struct PotentialOp {
	static constexpr int B = B_, T = T_, J = J_, NP = 1, NC = 1;
	using Elem = epos4;
	const epos4* pos;
	double xi[B], yi[B], zi[B], phi[B];

	__device__ const Elem* jsrc(int) const { return pos; }

	__device__ void begin(int64_t ibase, int tid)
	{
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const epos4 p = pos[ibase + tid + k * T];
			xi[k] = p.x;
			yi[k] = p.y;
			zi[k] = p.z;
			phi[k] = 0.0;
		}
	}

	__device__ void tile(const Elem* const* s)
	{
		const epos4* sj = s[0];
#pragma unroll 2
		for (int j = 0; j < J; ++j) {
			const epos4 pj = sj[j];
#pragma unroll
			for (int k = 0; k < B; ++k) {
				const double dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
				const double r2 = dx * dx + dy * dy + dz * dz;
				phi[k] += (r2 > 0.0) ? pj.w * rsqrt(r2) : 0.0;
			}
		}
	}

	__device__ void store(double* out, int tid)
	{
#pragma unroll
		for (int k = 0; k < B; ++k) out[tid + k * T] = phi[k];
	}
};

template <int B, int T, int J>
__global__ void __launch_bounds__(T) potential_kernel(const grav_batch b)
{
	PotentialOp<B, T, J> op;
	op.pos = static_cast<const epos4*>(b.pos);
	run_pairs(b, op);
}

__global__ void __launch_bounds__(256) energy_reduce_kernel(const grav_batch b, double* out)
{
	const int u = blockIdx.x;
	const grav_univ_desc U = b.univ[u];
	const int IT = b.tile.bpt * b.tile.threads;
	double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
	for (int il = threadIdx.x; il < U.n; il += blockDim.x) {
		const int64_t g = U.pad_off + il;
		const int64_t seg = g / IT;
		const int li = static_cast<int>(g - seg * IT);
		const grav_seg_desc S = b.seg[seg];
		double phi = 0.0;
		for (int k = 0; k < S.nslots; ++k) phi += b.part[static_cast<int64_t>(S.slot_base + k) * IT + li];
		const int64_t row = U.body_off + il;
		const double gm = b.r[4 * row + 3];
		const double vx = b.v[4 * row], vy = b.v[4 * row + 1], vz = b.v[4 * row + 2];
		acc[0] += 0.5 * gm * (vx * vx + vy * vy + vz * vz);
		acc[1] += -0.5 * gm * phi;
		acc[2] += gm * vx;
		acc[3] += gm * vy;
		acc[4] += gm * vz;
	}
	__shared__ double red[5][256];
#pragma unroll
	for (int c = 0; c < 5; ++c) red[c][threadIdx.x] = acc[c];
	__syncthreads();
	for (int w = 128; w > 0; w >>= 1) {
		if (threadIdx.x < w) {
#pragma unroll
			for (int c = 0; c < 5; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
		}
		__syncthreads();
	}
	if (threadIdx.x < 8) out[8 * u + threadIdx.x] = threadIdx.x < 5 ? red[threadIdx.x][0] : 0.0;
}

struct PotKernel {
	int bpt, threads, jtile;
	const void* fn;
	int smem;
};

#define GRAV_POT_ENTRY(B, T, J) \
	{B, T, J, reinterpret_cast<const void*>(&potential_kernel<B, T, J>), \
		pairs_smem_bytes<PotentialOp<B, T, J>>()}

static const PotKernel k_pot[] = {
	GRAV_POT_ENTRY(1, 128, 128), GRAV_POT_ENTRY(2, 128, 128), GRAV_POT_ENTRY(4, 128, 128),
	GRAV_POT_ENTRY(4, 128, 256), GRAV_POT_ENTRY(8, 128, 256), GRAV_POT_ENTRY(2, 256, 256),
	GRAV_POT_ENTRY(4, 256, 256), GRAV_POT_ENTRY(8, 256, 256), GRAV_POT_ENTRY(1, 256, 128),
	GRAV_POT_ENTRY(2, 256, 128),
};

int record_error(int code, const char* msg);

}  // namespace grav

extern "C" int grav_energy(const grav_batch* b, double* out, void* stream)
{
	using namespace grav;
	if (!b || !out) return record_error(GRAV_E_ARG, "NULL batch or out");
	if (b->mode != GRAV_MODE_FP64)
		return record_error(GRAV_E_ARG, "grav_energy needs an FP64-mode batch (double4 positions)");
	if (b->n_univ <= 0) return GRAV_OK;
	if (!b->univ || !b->seg || !b->pos || !b->r || !b->v || !b->part || !b->err)
		return record_error(GRAV_E_ARG, "NULL device pointer in grav_batch");
	const PotKernel* k = nullptr;
	for (const PotKernel& e : k_pot)
		if (e.bpt == b->tile.bpt && e.threads == b->tile.threads && e.jtile == b->tile.jtile) k = &e;
	if (!k) return record_error(GRAV_E_TILE, "tile shape has no potential kernel");
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	if (b->n_units > 0) {
		if (b->tile.grid <= 0 || b->tile.grid > b->n_units)
			return record_error(GRAV_E_ARG, "tile.grid must be in [1, n_units]");
		grav_batch copy = *b;
		void* args[] = {&copy};
		cudaError_t e = cudaLaunchKernel(k->fn, dim3(b->tile.grid), dim3(k->threads), args, k->smem, st);
		if (e != cudaSuccess) return record_error(GRAV_E_CUDA, cudaGetErrorString(e));
	}
	energy_reduce_kernel<<<b->n_univ, 256, 0, st>>>(*b, out);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return record_error(GRAV_E_CUDA, cudaGetErrorString(e));
	return GRAV_OK;
}
