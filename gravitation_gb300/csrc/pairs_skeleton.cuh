// pairs_skeleton.cuh -- persistent all-pairs loop shared by the diagnostic and adjoint
// kernels (the stage-1 kernels in stage1_f32.cu / stage1_f64.cu use the same scheme,
// written out by hand).
//
// The work list and its assignment are those of grav_plan: CTA c of the persistent
// grid walks units [c*U/G, (c+1)*U/G) of the flattened (segment, j-tile) list.  For
// each piece of a segment it asks the operation to load its i-bodies, streams the
// j-tiles of the universe through two shared-memory buffers with 1-D bulk copies
// (completion on an mbarrier, waits bounded in time), lets the operation consume each
// tile, and finally has it write NC FP64 values per i-body into the CTA's slot of
// b.part (layout [slot][NC][itile]).  A wait that expires sets GRAV_DEV_TIMEOUT in
// b.err and the CTA returns after one more bounded wait for the copy in flight.
//
// An operation type Op provides
//   static constexpr int B, T, J, NP, NC;      bodies/thread, threads, j-tile, arrays, outputs
//   using Elem;                                 element type of the j arrays (16 or 32 bytes)
//   const Elem* jsrc(int a) const;              base of padded array a (row 0 of the batch)
//   void begin(int64_t ibase, int tid);         load the i-bodies of rows ibase+tid+k*T
//   void tile(const Elem* const* s);            consume one tile (s[a] = array a, J rows)
//   void store(double* out, int tid);           out[c*IT + tid + k*T] for c < NC, k < B
#pragma once

#include "grav_device.cuh"

namespace grav {

template <class Op>
__device__ __forceinline__ void run_pairs(const grav_batch& b, Op& op)
{
	constexpr int B = Op::B, T = Op::T, J = Op::J, NP = Op::NP, NC = Op::NC;
	constexpr int IT = B * T;
	using E = typename Op::Elem;
	constexpr uint32_t TILE_BYTES = J * sizeof(E);
	static_assert(sizeof(E) % 16 == 0, "bulk copies move multiples of 16 bytes");
	extern __shared__ __align__(128) unsigned char pairs_smem[];
	E* tiles = reinterpret_cast<E*>(pairs_smem);  // [2 buffers][NP][J]
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

	int s = find_segment(b.seg, b.n_seg, ub);
	// positions, u and slots belong to the kernels before this one
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

		if (tid == 0) {
			const int bs = gt & 1;
			mbar_arrive_expect_tx(&bar[bs], NP * TILE_BYTES);
#pragma unroll
			for (int a = 0; a < NP; ++a)
				bulk_g2s(tiles + (bs * NP + a) * J, op.jsrc(a) + Uu.pad_off + jt0 * J, TILE_BYTES,
					&bar[bs]);
		}
		op.begin(Uu.pad_off + S.il0, tid);

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
#pragma unroll
				for (int a = 0; a < NP; ++a)
					bulk_g2s(tiles + (bn * NP + a) * J, op.jsrc(a) + Uu.pad_off + jt * J,
						TILE_BYTES, &bar[bn]);
			}
			const E* sp[NP];
#pragma unroll
			for (int a = 0; a < NP; ++a) sp[a] = tiles + (bs * NP + a) * J;
			op.tile(sp);
		}
		if (timed_out) break;

		const int64_t slot = S.slot_base + (c - S.cta_first);
		op.store(b.part + slot * NC * IT, tid);
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

template <class Op>
constexpr int pairs_smem_bytes()
{
	return 2 * Op::NP * Op::J * static_cast<int>(sizeof(typename Op::Elem));
}

}  // namespace grav
