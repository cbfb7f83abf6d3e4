// stage1_sym.cu -- stage 1 over unique pairs (GRAV_MODE_FP32U, GRAV_MODE_FP32CU,
// GRAV_MODE_FP32UN).
//
// The reference's CPU kernels visit every unordered pair once and update both bodies
// (np1.py:81-95, _lib1_/lib.c:78-114, _lib4_/lib.c:244-317: a_i -= ..., a_j += ...).
// This kernel does the same on the GPU, which removes a third of the FMA-pipe work of
// the all-pairs kernel (16 instead of 2 x 12 FMA-pipe operations per pair).  Arithmetic
// per pair is the FP32 law of stage1_f32.cu:
//     d = r_j - r_i ; r2 = |d|^2 + eps2 ; inv3 = rsqrt(r2)^3
//     a_i += (Gm_j inv3) d ;  a_j -= (Gm_i inv3) d
//
// Decomposition (plan: grav_plan_pairs).  Each universe is cut into row blocks of R =
// 32 * W * B bodies (one segment each); the work units of row block I are the j-tiles
// (JT bodies) of blocks J >= I.  A j-tile inside block I itself is done "all pairs,
// rows only" (every ordered pair of the block once, like stage1_f32.cu); a j-tile of a
// block J > I is done on unique pairs: warp w holds 32 x B rows of block I, and for
// each 32-body chunk of the tile, lane l meets body (l + s) mod 32 of the chunk at step
// s while the chunk's column sums rotate one lane per step (shfl), so after 32 steps
// every row of the warp has met every body of the chunk once and each lane holds the
// complete column sum of "its" body.  Each warp writes its column sums to its own row of
// a shared-memory buffer, and the tile's column sums (the warps added in a fixed order)
// go into the column slot of (I, J): block J's segment lists its row slots first and then
// one column slot per block I < J (its last J slots), so stage 2 adds them like any
// partial sums (fixed order: the result does not depend on scheduling).
// Row sums are FP32 per tile, folded into compensated (TwoSum) FP32 hi+lo sums, as in
// stage1_f32.cu, and go out as FP32 (hi, lo) pairs; column sums are FP32 per tile and go
// out as FP32 (the first 3R floats of the slot), which stage 2 adds by TwoSum in FP32.
#include "grav_device.cuh"

namespace grav {

// KIND selects the separations:
//   SYM_PLAIN (GRAV_MODE_FP32U): FP32 positions, d = hi_j - hi_i.
//   SYM_DS    (GRAV_MODE_FP32CU): FP32 hi and lo parts of the FP64 positions,
//             d = (hi_j - hi_i) + (lo_j - lo_i), exact to FP32 relative precision however
//             far from the origin the bodies are (+6 FADD per pair).
//   SYM_NEAR  (GRAV_MODE_FP32UN): the SYM_PLAIN loop plus one compare per pair against
//             the near radius (grav_device.cuh, near_threshold); a step of the loop where
//             any lane of the warp met a near pair re-evaluates those pairs from the
//             double-single separation and adds the difference (near_delta).  Near pairs
//             are rare (~3e-5 of the pairs of the N = 65536 uniform cube), so this path is
//             cold; it is warp-uniform, so it costs no divergence.
enum { SYM_PLAIN = 0, SYM_DS = 1, SYM_NEAR = 2 };

template <int B, int W, int JT, int UNROLL = 4, int KIND = SYM_PLAIN>
__global__ void __launch_bounds__(32 * W) stage1_sym_kernel(const grav_batch b)
{
	constexpr int T = 32 * W;
	constexpr int R = T * B;            // rows per block (= itile)
	constexpr int TPB = R / JT;         // j-tiles per block
	constexpr int NCH = JT / 32;        // 32-body chunks per j-tile
	constexpr uint32_t TILE_BYTES = JT * sizeof(float4);
	constexpr int NP = KIND == SYM_PLAIN ? 1 : 2;   // position arrays copied per j-tile
	constexpr bool DS = KIND == SYM_DS;             // double-single separations everywhere
	constexpr bool NEAR = KIND == SYM_NEAR;         // double-single for near pairs only
	static_assert(R % JT == 0 && JT % 32 == 0, "tile shapes");
	extern __shared__ __align__(128) float4 sym_tiles[];   // [2 buffers][NP][JT]
	// column sums of a j-tile, one row per warp: every warp writes each chunk of the tile
	// once, and the flush adds the warps in a fixed order (no shared-memory atomics, whose
	// order would depend on warp timing)
	__shared__ float colacc[W][3][JT];
	__shared__ __align__(8) uint64_t bar[2];
	// low parts of this thread's rows (NEAR): read only on the cold correction path, by
	// the thread that wrote them ([k][tid]: conflict-free 16-byte accesses)
	__shared__ float4 rowlo[NEAR ? B : 1][NEAR ? T : 1];
	// NEAR with 8 rows per thread keeps the compensated row sums (hi, lo) in shared memory
	// instead of 48 registers, touched once per j-tile: the cold correction path's
	// registers would otherwise cost a resident CTA per SM
	constexpr bool SS = NEAR && B >= 8;
	__shared__ float2 csum[SS ? 3 : 1][SS ? B : 1][SS ? T : 1];

	const int tid = threadIdx.x;
	const int lane = tid & 31;
	const int warp = tid >> 5;
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

	const float4* __restrict__ pos = static_cast<const float4*>(b.pos);
	const float eps2 = b.eps2;

	// Segment of unit ub by bisection, and no programmatic-launch instructions: this
	// kernel runs for 1e5-1e6 cycles per CTA, where a few microseconds of prologue do
	// not matter, and with the warp-parallel search or griddepcontrol in it the
	// compiled main loop measured 1-4 % slower on GB300 (N = 65536, tile 8/128/256).
	int s;
	{
		int lo = 0, hi = b.n_seg - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (b.seg[mid].unit_begin <= ub) lo = mid;
			else hi = mid - 1;
		}
		s = lo;
	}

	uint32_t gt = 0;
	bool timed_out = false;
	while (ub < ue && s < b.n_seg) {
		const grav_seg_desc S = b.seg[s];
		if (S.n_units == 0 || S.unit_begin + S.n_units <= ub) {
			++s;
			continue;
		}
		const grav_univ_desc Uu = b.univ[S.u];
		const int blkI = S.il0 / R;
		const int64_t t0 = ub - S.unit_begin;                              // local unit
		const int64_t t1 = min(ue - S.unit_begin, (int64_t)S.n_units);
		const int nt = static_cast<int>(t1 - t0);
		const int64_t jt_first = static_cast<int64_t>(blkI) * TPB;       // global j-tile of unit 0
		const float4* __restrict__ jsrc = pos + Uu.pad_off;
		const float4* __restrict__ jsrclo = pos + b.n_pad_total + Uu.pad_off;

		if (tid == 0) {
			const int bs = gt & 1;
			mbar_arrive_expect_tx(&bar[bs], NP * TILE_BYTES);
			bulk_g2s(sym_tiles + bs * NP * JT, jsrc + (jt_first + t0) * JT, TILE_BYTES, &bar[bs]);
			if (NP == 2)
				bulk_g2s(sym_tiles + (bs * NP + 1) * JT, jsrclo + (jt_first + t0) * JT, TILE_BYTES,
					&bar[bs]);
		}

		// rows of this warp: w*32*B + k*32 + lane
		const int64_t ibase = Uu.pad_off + S.il0 + warp * 32 * B + lane;
		float xi[B], yi[B], zi[B], gi[B], fx[B], fy[B], fz[B];
		float xl[B], yl[B], zl[B];                       // low parts (DS)
		float hx[B], hy[B], hz[B], lx[B], ly[B], lz[B];  // compensated row sums
		float xmax = 0.f;                                // NEAR: largest |coordinate| of the rows
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const float4 p = pos[ibase + k * 32];
			xi[k] = p.x;
			yi[k] = p.y;
			zi[k] = p.z;
			gi[k] = p.w;
			if (DS) {
				const float4 q = pos[b.n_pad_total + ibase + k * 32];
				xl[k] = q.x;
				yl[k] = q.y;
				zl[k] = q.z;
			} else {
				xl[k] = yl[k] = zl[k] = 0.f;
			}
			if (NEAR) {
				rowlo[NEAR ? k : 0][NEAR ? tid : 0] = pos[b.n_pad_total + ibase + k * 32];
				xmax = fmaxf(xmax, near_scale(p.x, p.y, p.z));
			}
			fx[k] = fy[k] = fz[k] = 0.f;
			hx[k] = hy[k] = hz[k] = lx[k] = ly[k] = lz[k] = 0.f;
			if (SS) {
#pragma unroll
				for (int cpt = 0; cpt < 3; ++cpt) csum[SS ? cpt : 0][SS ? k : 0][SS ? tid : 0] = make_float2(0.f, 0.f);
			}
		}
		const float thr = near_threshold(xmax);

		for (int t = 0; t < nt; ++t, ++gt) {
			const int bs = gt & 1;
			const bool ok = mbar_wait_bounded(&bar[bs], (gt >> 1) & 1);
			if (__syncthreads_or(!ok)) {
				timed_out = true;
				break;
			}
			const int64_t jt = jt_first + t0 + t;  // global j-tile index in the universe
			if (tid == 0 && t + 1 < nt) {
				const int bn = (gt + 1) & 1;
				mbar_arrive_expect_tx(&bar[bn], NP * TILE_BYTES);
				bulk_g2s(sym_tiles + bn * NP * JT, jsrc + (jt + 1) * JT, TILE_BYTES, &bar[bn]);
				if (NP == 2)
					bulk_g2s(sym_tiles + (bn * NP + 1) * JT, jsrclo + (jt + 1) * JT, TILE_BYTES,
						&bar[bn]);
			}
			const float4* __restrict__ sj = sym_tiles + bs * NP * JT;
			const float4* __restrict__ sjl = sj + JT;  // low parts (NP == 2)
			const int blkJ = static_cast<int>(jt / TPB);
			if (blkJ == blkI) {
				// diagonal block: every ordered pair of the block once, rows only.  In NEAR
				// mode a tile that holds this warp's own rows meets their self pairs (d = 0,
				// r2 = eps2): there the near test also requires r2 > eps2, so that self pairs
				// do not send the warp down the correction path
				const int jl0 = static_cast<int>(jt - static_cast<int64_t>(blkI) * TPB) * JT;
				const bool own = jl0 < (warp + 1) * 32 * B && jl0 + JT > warp * 32 * B;
#pragma unroll 4
				for (int j = 0; j < JT; ++j) {
					const float4 pj = sj[j];
					float4 lj = make_float4(0.f, 0.f, 0.f, 0.f);
					if (DS) lj = sjl[j];
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
						if (NEAR) near |= own ? (r2 < thr) & (r2 > eps2) : (r2 < thr);
						const float inv = rsqrt_sfu(r2);
						float w = pj.w * inv;
						w = w * (inv * inv);
						fx[k] = fmaf(dx, w, fx[k]);
						fy[k] = fmaf(dy, w, fy[k]);
						fz[k] = fmaf(dz, w, fz[k]);
					}
					if (NEAR && __any_sync(0xffffffffu, near)) {
						lj = sjl[j];
#pragma unroll
						for (int k = 0; k < B; ++k) {
							const float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
							const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
							const bool nk = (r2 < thr) & (r2 > eps2);
							if (__any_sync(0xffffffffu, nk)) {
								float ex, ey, ez;
								near_delta(dx, dy, dz, r2, lj, rowlo[NEAR ? k : 0][NEAR ? tid : 0],
									eps2, nk, ex, ey, ez);
								fx[k] = fmaf(ex, pj.w, fx[k]);
								fy[k] = fmaf(ey, pj.w, fy[k]);
								fz[k] = fmaf(ez, pj.w, fz[k]);
							}
						}
					}
				}
			} else {
				// unique pairs with block J > I: rotate the chunk's column sums
#pragma unroll 1
				for (int cc = 0; cc < NCH; ++cc) {
					const int ch = (cc + warp) & (NCH - 1);
					const float4* __restrict__ sc = sj + ch * 32;
					const float4* __restrict__ scl = sjl + ch * 32;
					float cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll UNROLL
					for (int st = 0; st < 32; ++st) {
						const float4 pj = sc[(lane + st) & 31];
						float4 lj = make_float4(0.f, 0.f, 0.f, 0.f);
						if (DS) lj = scl[(lane + st) & 31];
						float rmin = 0.f, rprev = 0.f;   // NEAR: smallest r2 of this step
#pragma unroll
						for (int k = 0; k < B; ++k) {
							float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
							if (DS) {
								dx = dx + (lj.x - xl[k]);
								dy = dy + (lj.y - yl[k]);
								dz = dz + (lj.z - zl[k]);
							}
							const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
							if (NEAR) near_min_step<B>(k, r2, rmin, rprev);
							const float inv = rsqrt_sfu(r2);
							const float inv3 = inv * (inv * inv);
							const float wj = pj.w * inv3;
							const float wi = gi[k] * inv3;
							fx[k] = fmaf(dx, wj, fx[k]);
							fy[k] = fmaf(dy, wj, fy[k]);
							fz[k] = fmaf(dz, wj, fz[k]);
							cx = fmaf(-dx, wi, cx);
							cy = fmaf(-dy, wi, cy);
							cz = fmaf(-dz, wi, cz);
						}
						if (NEAR && __any_sync(0xffffffffu, rmin < thr)) {
							// cold path: the pairs of this step closer than the near radius
							// again, from the double-single separation (row and column)
							lj = scl[(lane + st) & 31];
#pragma unroll
							for (int k = 0; k < B; ++k) {
								const float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
								const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
								const bool nk = (r2 < thr) & (r2 > eps2);
								if (__any_sync(0xffffffffu, nk)) {
									float ex, ey, ez;
									near_delta(dx, dy, dz, r2, lj,
										rowlo[NEAR ? k : 0][NEAR ? tid : 0], eps2, nk, ex, ey, ez);
									fx[k] = fmaf(ex, pj.w, fx[k]);
									fy[k] = fmaf(ey, pj.w, fy[k]);
									fz[k] = fmaf(ez, pj.w, fz[k]);
									cx = fmaf(-ex, gi[k], cx);
									cy = fmaf(-ey, gi[k], cy);
									cz = fmaf(-ez, gi[k], cz);
								}
							}
						}
						const int src = (lane + 1) & 31;
						cx = __shfl_sync(0xffffffffu, cx, src);
						cy = __shfl_sync(0xffffffffu, cy, src);
						cz = __shfl_sync(0xffffffffu, cz, src);
					}
					colacc[warp][0][ch * 32 + lane] = cx;
					colacc[warp][1][ch * 32 + lane] = cy;
					colacc[warp][2][ch * 32 + lane] = cz;
				}
				__syncthreads();
				// column sums of this tile -> column slot of (I, J), the warps added in order.
				// They are FP32 sums, so they go out as FP32 (first half of the slot; stage
				// 2 adds them by TwoSum in FP32): half the bytes of an FP64 slot
				const int sJ = s + (blkJ - blkI);
				const grav_seg_desc SJ = b.seg[sJ];
				const int64_t slot = SJ.slot_base + SJ.nslots - (blkJ - blkI);
				float* __restrict__ out = reinterpret_cast<float*>(b.part + slot * 3 * R) +
					(jt * JT - static_cast<int64_t>(blkJ) * R);
				for (int i = tid; i < JT; i += T) {
					float sx = colacc[0][0][i], sy = colacc[0][1][i], sz = colacc[0][2][i];
#pragma unroll
					for (int w = 1; w < W; ++w) {
						sx += colacc[w][0][i];
						sy += colacc[w][1][i];
						sz += colacc[w][2][i];
					}
					out[i] = sx;
					out[R + i] = sy;
					out[2 * R + i] = sz;
				}
			}
#pragma unroll
			for (int k = 0; k < B; ++k) {
				if (SS) {
					float2* cs = &csum[0][SS ? k : 0][SS ? tid : 0];
					constexpr int CS = SS ? B * T : 0;   // stride between components
					float2 h0 = cs[0], h1 = cs[CS], h2 = cs[2 * CS];
					two_sum_acc(h0.x, h0.y, fx[k]);
					two_sum_acc(h1.x, h1.y, fy[k]);
					two_sum_acc(h2.x, h2.y, fz[k]);
					cs[0] = h0;
					cs[CS] = h1;
					cs[2 * CS] = h2;
				} else {
					two_sum_acc(hx[k], lx[k], fx[k]);
					two_sum_acc(hy[k], ly[k], fy[k]);
					two_sum_acc(hz[k], lz[k], fz[k]);
				}
				fx[k] = fy[k] = fz[k] = 0.f;
			}
		}
		if (timed_out) break;

		// row sums of this CTA's piece as FP32 (hi, lo) pairs, one 8-byte slot entry each
		const int64_t slot = S.slot_base + (c - S.cta_first);
		float2* __restrict__ out = reinterpret_cast<float2*>(b.part + slot * 3 * R);
		const int r0 = warp * 32 * B + lane;
#pragma unroll
		for (int k = 0; k < B; ++k) {
			if (SS) {
				out[r0 + k * 32] = csum[0][SS ? k : 0][SS ? tid : 0];
				out[R + r0 + k * 32] = csum[SS ? 1 : 0][SS ? k : 0][SS ? tid : 0];
				out[2 * R + r0 + k * 32] = csum[SS ? 2 : 0][SS ? k : 0][SS ? tid : 0];
			} else {
				out[r0 + k * 32] = make_float2(hx[k], lx[k]);
				out[R + r0 + k * 32] = make_float2(hy[k], ly[k]);
				out[2 * R + r0 + k * 32] = make_float2(hz[k], lz[k]);
			}
		}
		ub = S.unit_begin + t1;
		++s;
	}

	if (timed_out && tid == 0) {
		set_error(b.err, GRAV_DEV_TIMEOUT);
		mbar_wait_bounded(&bar[gt & 1], (gt >> 1) & 1);
	}
}

// launched the ordinary way (not as a programmatic dependent): see the kernel's prologue
#define GRAV_SYM_ENTRY(B, W, J) \
	{GRAV_MODE_FP32U, B, 32 * W, J, \
		reinterpret_cast<const void*>(&stage1_sym_kernel<B, W, J, 4, SYM_PLAIN>), 2 * J * 16, false}
#define GRAV_SYMC_ENTRY(B, W, J) \
	{GRAV_MODE_FP32CU, B, 32 * W, J, \
		reinterpret_cast<const void*>(&stage1_sym_kernel<B, W, J, 4, SYM_DS>), 2 * 2 * J * 16, false}
// the near kernel's step loop is not unrolled: with its vote and cold path in every step
// the unrolled form held 167 registers against 147 and ran 1.4 % slower (N = 65536,
// tile 8/128/256: stage 1 1.458 against 1.438 ms; unrolled by 2 1.456, by 8 it spilled)
#define GRAV_SYMN_ENTRY(B, W, J) \
	{GRAV_MODE_FP32UN, B, 32 * W, J, \
		reinterpret_cast<const void*>(&stage1_sym_kernel<B, W, J, 1, SYM_NEAR>), 2 * 2 * J * 16, false}

static const Stage1Kernel k_table_sym[] = {
	GRAV_SYM_ENTRY(4, 4, 128),
	GRAV_SYM_ENTRY(4, 8, 256),
	GRAV_SYM_ENTRY(8, 4, 256),
	GRAV_SYM_ENTRY(4, 4, 256),
	GRAV_SYM_ENTRY(2, 8, 256),
	GRAV_SYM_ENTRY(8, 8, 256),
	GRAV_SYM_ENTRY(8, 4, 128),
	GRAV_SYM_ENTRY(8, 4, 64),
	GRAV_SYM_ENTRY(4, 2, 64),
	GRAV_SYMC_ENTRY(4, 4, 128),
	GRAV_SYMC_ENTRY(8, 4, 256),
	GRAV_SYMC_ENTRY(4, 4, 256),
	GRAV_SYMC_ENTRY(4, 8, 256),
	GRAV_SYMN_ENTRY(4, 4, 128),
	GRAV_SYMN_ENTRY(8, 4, 256),
	GRAV_SYMN_ENTRY(8, 4, 128),
	GRAV_SYMN_ENTRY(8, 4, 64),
	GRAV_SYMN_ENTRY(4, 4, 256),
	GRAV_SYMN_ENTRY(4, 8, 256),
	GRAV_SYMN_ENTRY(4, 2, 64),
	GRAV_SYMN_ENTRY(8, 2, 64),
	GRAV_SYMN_ENTRY(8, 2, 128),
};

int stage1_table_sym(const Stage1Kernel** out)
{
	*out = k_table_sym;
	return static_cast<int>(sizeof(k_table_sym) / sizeof(k_table_sym[0]));
}

}  // namespace grav
