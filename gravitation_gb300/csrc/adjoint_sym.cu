// adjoint_sym.cu -- the backward pair kernel over unique pairs.
//
// Same transposed step as adjoint.cu (derivation there), with each unordered pair (i, j)
// visited once.  For d = r_j - r_i, inv3 = |d|^-3, inv2 = |d|^-2 (both 0 at zero
// separation), ci = Gm_j inv3, cj = Gm_i inv3 and t5 = (cj (d.u_j) - ci (d.u_i)) inv2
// (= (Gm_i d.u_j - Gm_j d.u_i) / |d|^5):
//   row i    a_i += ci d                   h_i: P += inv3 u_j, S += ci, Q += t5 d
//            g_i += inv3 (d.u_j)           (h_i = Gm_i P - u_i S - 3 Q, formed per tile)
//   column j a_j -= cj d                   h_j += ci u_i - cj u_j + 3 t5 d
//            g_j -= inv3 (d.u_i)
// since Jf(-d) = Jf(d) (Jf(d) = I/|d|^3 - 3 d d^T/|d|^5) and the pair's h terms for j are
// those for i with the roles of the bodies swapped.  With the accelerations (FA = true:
// the forward's a_k is recomputed here) that is 46 FMA-pipe operations and one MUFU per
// unordered pair, against 2 x 33 when both ordered pairs are visited; when the caller
// keeps the forward's accelerations (FA = false) the a terms drop out: 40 operations and
// 4 rotating column values instead of 7.
//
// Decomposition: the plan of grav_plan_pairs and the warp scheme of stage1_sym.cu.  Row
// block I's units are the j-tiles of blocks J >= I; a j-tile of block I itself is done
// with every ordered pair, rows only; a j-tile of a block J > I on unique pairs: lane l
// meets body (l + s) mod 32 of a 32-body chunk at step s while the chunk's column
// values rotate one lane per step, then each warp writes them to its own row of a
// shared-memory buffer, and the tile's column sums (the warps added in a fixed order) go,
// as FP32, to the column slot of (I, J) (block J's last J slots).  Row
// sums are compensated FP32 (TwoSum) and go out as FP32 (hi, lo) pairs.  Slot layout
// [slot][NC][R]: a, h, g (NC = 7) or h, g (NC = 4).
#include <mutex>
#include <set>
#include <utility>

#include "grav_device.cuh"

namespace grav {

int record_error(int code, const char* msg);

template <int B, int W, int JT, bool FA>
__global__ void __launch_bounds__(32 * W) vjp_sym_kernel(const grav_batch b,
	const float4* __restrict__ upos)
{
	constexpr int T = 32 * W;
	constexpr int R = T * B;      // rows per block (= itile)
	constexpr int TPB = R / JT;   // j-tiles per block
	constexpr int NCH = JT / 32;  // 32-body chunks per j-tile
	constexpr int NC = FA ? 7 : 4;  // [a (3),] h (3), g
	constexpr int H0 = FA ? 3 : 0;  // first h component of a slot
	constexpr int G0 = H0 + 3;      // the g component
	constexpr uint32_t TILE_BYTES = JT * sizeof(float4);
	static_assert(R % JT == 0 && JT % 32 == 0 && (NCH & (NCH - 1)) == 0, "tile shapes");
	extern __shared__ __align__(128) float4 vs_tiles[];  // [2 buffers][pos, u][JT]
	// column sums of a j-tile, one row per warp, added over the warps in a fixed order
	// at the flush (no shared-memory atomics, whose order would depend on warp timing)
	__shared__ float colacc[W][NC][JT];
	__shared__ __align__(8) uint64_t bar[2];
	// with 4 rows per thread the compensated row sums (hi, lo) live in shared memory,
	// touched once per j-tile, instead of 20 registers per row: 128 instead of 168
	// registers with the accelerations recomputed, a fourth resident CTA per SM
	constexpr bool SS = B >= 4;
	__shared__ float2 csum[SS ? NC : 1][SS ? B : 1][SS ? T : 1];

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
		const int blkI = S.il0 / R;
		const int64_t t0 = ub - S.unit_begin;
		const int64_t t1 = min(ue - S.unit_begin, (int64_t)S.n_units);
		const int nt = static_cast<int>(t1 - t0);
		const int64_t jt_first = static_cast<int64_t>(blkI) * TPB;
		const float4* __restrict__ jpos = pos + Uu.pad_off;
		const float4* __restrict__ ju = upos + Uu.pad_off;

		if (tid == 0) {
			const int bs = gt & 1;
			mbar_arrive_expect_tx(&bar[bs], 2 * TILE_BYTES);
			bulk_g2s(vs_tiles + (bs * 2) * JT, jpos + (jt_first + t0) * JT, TILE_BYTES, &bar[bs]);
			bulk_g2s(vs_tiles + (bs * 2 + 1) * JT, ju + (jt_first + t0) * JT, TILE_BYTES, &bar[bs]);
		}

		// rows of this warp: w*32*B + k*32 + lane
		const int64_t ibase = Uu.pad_off + S.il0 + warp * 32 * B + lane;
		float xi[B], yi[B], zi[B], gi[B], uxi[B], uyi[B], uzi[B];
		float fa[3][B], fp[3][B], fq[3][B], fs[B], fg[B];                // per tile
		float ah[3][B], al[3][B], hh[3][B], hl[3][B], gh[B], gl[B];   // compensated
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const float4 p = pos[ibase + k * 32];
			const float4 q = upos[ibase + k * 32];
			xi[k] = p.x;
			yi[k] = p.y;
			zi[k] = p.z;
			gi[k] = p.w;
			uxi[k] = q.x;
			uyi[k] = q.y;
			uzi[k] = q.z;
#pragma unroll
			for (int q3 = 0; q3 < 3; ++q3) {
				fa[q3][k] = fp[q3][k] = fq[q3][k] = 0.f;
				ah[q3][k] = al[q3][k] = hh[q3][k] = hl[q3][k] = 0.f;
			}
			fs[k] = fg[k] = gh[k] = gl[k] = 0.f;
			if (SS) {
#pragma unroll
				for (int q = 0; q < NC; ++q) csum[SS ? q : 0][SS ? k : 0][SS ? tid : 0] = make_float2(0.f, 0.f);
			}
		}

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
				mbar_arrive_expect_tx(&bar[bn], 2 * TILE_BYTES);
				bulk_g2s(vs_tiles + (bn * 2) * JT, jpos + (jt + 1) * JT, TILE_BYTES, &bar[bn]);
				bulk_g2s(vs_tiles + (bn * 2 + 1) * JT, ju + (jt + 1) * JT, TILE_BYTES, &bar[bn]);
			}
			const float4* __restrict__ sp = vs_tiles + (bs * 2) * JT;
			const float4* __restrict__ su = sp + JT;
			const int blkJ = static_cast<int>(jt / TPB);
			if (blkJ == blkI) {
				// diagonal block: every ordered pair of the block once, rows only
#pragma unroll 2
				for (int j = 0; j < JT; ++j) {
					const float4 pj = sp[j];
					const float4 uj = su[j];
#pragma unroll
					for (int k = 0; k < B; ++k) {
						const float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
						const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
						const float inv = (r2 > 0.f) ? rsqrt_sfu(r2) : 0.f;
						const float inv2 = inv * inv;
						const float inv3 = inv2 * inv;
						const float inv5 = inv3 * inv2;
						const float ci = pj.w * inv3;
						if constexpr (FA) {
							fa[0][k] = fmaf(ci, dx, fa[0][k]);
							fa[1][k] = fmaf(ci, dy, fa[1][k]);
							fa[2][k] = fmaf(ci, dz, fa[2][k]);
						}
						fs[k] += ci;
						fp[0][k] = fmaf(uj.x, inv3, fp[0][k]);
						fp[1][k] = fmaf(uj.y, inv3, fp[1][k]);
						fp[2][k] = fmaf(uj.z, inv3, fp[2][k]);
						const float duj = fmaf(dz, uj.z, fmaf(dy, uj.y, dx * uj.x));
						const float dui = fmaf(dz, uzi[k], fmaf(dy, uyi[k], dx * uxi[k]));
						const float t5 = fmaf(gi[k], duj, -pj.w * dui) * inv5;
						fq[0][k] = fmaf(t5, dx, fq[0][k]);
						fq[1][k] = fmaf(t5, dy, fq[1][k]);
						fq[2][k] = fmaf(t5, dz, fq[2][k]);
						fg[k] = fmaf(duj, inv3, fg[k]);
					}
				}
			} else {
				// unique pairs with block J > I: rotate the chunk's column values
#pragma unroll 1
				for (int cc = 0; cc < NCH; ++cc) {
					const int ch = (cc + warp) & (NCH - 1);
					const float4* __restrict__ cp = sp + ch * 32;
					const float4* __restrict__ cu = su + ch * 32;
					float cax = 0.f, cay = 0.f, caz = 0.f, chx = 0.f, chy = 0.f, chz = 0.f, cg = 0.f;
					// unrolled by 4 with the forces recomputed, by 2 without (measured at 8192
					// and 16384 bodies: 3 % faster / 1 % slower with 4 than with 2)
#pragma unroll (FA ? 4 : 2)
					for (int st = 0; st < 32; ++st) {
						const float4 pj = cp[(lane + st) & 31];
						const float4 uj = cu[(lane + st) & 31];
#pragma unroll
						for (int k = 0; k < B; ++k) {
							const float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
							const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
							const float inv = (r2 > 0.f) ? rsqrt_sfu(r2) : 0.f;
							const float inv2 = inv * inv;
							const float inv3 = inv2 * inv;
							const float ci = pj.w * inv3;   // Gm_j / r^3
							const float cj = gi[k] * inv3;  // Gm_i / r^3
							// row i
							if constexpr (FA) {
								fa[0][k] = fmaf(ci, dx, fa[0][k]);
								fa[1][k] = fmaf(ci, dy, fa[1][k]);
								fa[2][k] = fmaf(ci, dz, fa[2][k]);
							}
							fs[k] += ci;
							fp[0][k] = fmaf(uj.x, inv3, fp[0][k]);
							fp[1][k] = fmaf(uj.y, inv3, fp[1][k]);
							fp[2][k] = fmaf(uj.z, inv3, fp[2][k]);
							const float duj = fmaf(dz, uj.z, fmaf(dy, uj.y, dx * uj.x));
							const float dui = fmaf(dz, uzi[k], fmaf(dy, uyi[k], dx * uxi[k]));
							const float t5 = fmaf(cj, duj, -ci * dui) * inv2;
							fq[0][k] = fmaf(t5, dx, fq[0][k]);
							fq[1][k] = fmaf(t5, dy, fq[1][k]);
							fq[2][k] = fmaf(t5, dz, fq[2][k]);
							fg[k] = fmaf(duj, inv3, fg[k]);
							// column j
							if constexpr (FA) {
								cax = fmaf(-cj, dx, cax);
								cay = fmaf(-cj, dy, cay);
								caz = fmaf(-cj, dz, caz);
							}
							const float t3 = 3.f * t5;
							chx = fmaf(t3, dx, fmaf(-cj, uj.x, fmaf(ci, uxi[k], chx)));
							chy = fmaf(t3, dy, fmaf(-cj, uj.y, fmaf(ci, uyi[k], chy)));
							chz = fmaf(t3, dz, fmaf(-cj, uj.z, fmaf(ci, uzi[k], chz)));
							cg = fmaf(-dui, inv3, cg);
						}
						const int src = (lane + 1) & 31;
						if constexpr (FA) {
							cax = __shfl_sync(0xffffffffu, cax, src);
							cay = __shfl_sync(0xffffffffu, cay, src);
							caz = __shfl_sync(0xffffffffu, caz, src);
						}
						chx = __shfl_sync(0xffffffffu, chx, src);
						chy = __shfl_sync(0xffffffffu, chy, src);
						chz = __shfl_sync(0xffffffffu, chz, src);
						cg = __shfl_sync(0xffffffffu, cg, src);
					}
					const int ci0 = ch * 32 + lane;
					if constexpr (FA) {
						colacc[warp][0][ci0] = cax;
						colacc[warp][1][ci0] = cay;
						colacc[warp][2][ci0] = caz;
					}
					colacc[warp][H0][ci0] = chx;
					colacc[warp][H0 + 1][ci0] = chy;
					colacc[warp][H0 + 2][ci0] = chz;
					colacc[warp][G0][ci0] = cg;
				}
				__syncthreads();
				// column sums of this tile -> column slot of (I, J) as FP32, the warps added
				// in order
				const int sJ = s + (blkJ - blkI);
				const grav_seg_desc SJ = b.seg[sJ];
				const int64_t slot = SJ.slot_base + SJ.nslots - (blkJ - blkI);
				float* __restrict__ out = reinterpret_cast<float*>(b.part + slot * NC * R) +
					(jt * JT - static_cast<int64_t>(blkJ) * R);
				for (int i = tid; i < JT; i += T) {
#pragma unroll
					for (int q = 0; q < NC; ++q) {
						float sq = colacc[0][q][i];
#pragma unroll
						for (int w = 1; w < W; ++w) sq += colacc[w][q][i];
						out[q * R + i] = sq;
					}
				}
			}
			// fold the tile's row partials into the compensated sums
#pragma unroll
			for (int k = 0; k < B; ++k) {
				const float ui[3] = {uxi[k], uyi[k], uzi[k]};
#pragma unroll
				for (int q3 = 0; q3 < 3; ++q3) {
					// h = Gm_i P - u_i S - 3 Q
					const float ht = fmaf(gi[k], fp[q3][k], fmaf(-ui[q3], fs[k], -3.f * fq[q3][k]));
					if (SS) {
						if constexpr (FA) {
							float2 v = csum[SS ? q3 : 0][SS ? k : 0][SS ? tid : 0];
							two_sum_acc(v.x, v.y, fa[q3][k]);
							csum[SS ? q3 : 0][SS ? k : 0][SS ? tid : 0] = v;
						}
						float2 v = csum[SS ? H0 + q3 : 0][SS ? k : 0][SS ? tid : 0];
						two_sum_acc(v.x, v.y, ht);
						csum[SS ? H0 + q3 : 0][SS ? k : 0][SS ? tid : 0] = v;
					} else {
						if constexpr (FA) two_sum_acc(ah[q3][k], al[q3][k], fa[q3][k]);
						two_sum_acc(hh[q3][k], hl[q3][k], ht);
					}
					fa[q3][k] = fp[q3][k] = fq[q3][k] = 0.f;
				}
				if (SS) {
					float2 v = csum[SS ? G0 : 0][SS ? k : 0][SS ? tid : 0];
					two_sum_acc(v.x, v.y, fg[k]);
					csum[SS ? G0 : 0][SS ? k : 0][SS ? tid : 0] = v;
				} else {
					two_sum_acc(gh[k], gl[k], fg[k]);
				}
				fs[k] = fg[k] = 0.f;
			}
		}
		if (timed_out) break;

		// row sums of this CTA's piece as FP32 (hi, lo) pairs, one 8-byte entry each
		const int64_t slot = S.slot_base + (c - S.cta_first);
		float2* __restrict__ out = reinterpret_cast<float2*>(b.part + slot * NC * R);
		const int r0 = warp * 32 * B + lane;
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const int i = r0 + k * 32;
#pragma unroll
			if (SS) {
#pragma unroll
				for (int q = 0; q < NC; ++q) out[q * R + i] = csum[SS ? q : 0][SS ? k : 0][SS ? tid : 0];
			} else {
#pragma unroll
				for (int q3 = 0; q3 < 3; ++q3) {
					if constexpr (FA) out[q3 * R + i] = make_float2(ah[q3][k], al[q3][k]);
					out[(H0 + q3) * R + i] = make_float2(hh[q3][k], hl[q3][k]);
				}
				out[G0 * R + i] = make_float2(gh[k], gl[k]);
			}
		}
		ub = S.unit_begin + t1;
		++s;
	}

	// the next kernel in the stream may start launching now (it waits for this grid)
	grid_dep_launch();
	if (timed_out && tid == 0) {
		set_error(b.err, GRAV_DEV_TIMEOUT);
		// the copy that did not arrive is the only one in flight; give it one more
		// bounded wait so that it does not land in shared memory after this CTA exits
		mbar_wait_bounded(&bar[gt & 1], (gt >> 1) & 1);
	}
}

struct VjpSymKernel {
	int bpt, threads, jtile;
	bool fa;
	const void* fn;
	int smem;
};

#define GRAV_VJPSYM_ENTRY(B, W, J, FA) \
	{B, 32 * W, J, FA, reinterpret_cast<const void*>(&vjp_sym_kernel<B, W, J, FA>), 2 * 2 * J * 16}

static const VjpSymKernel k_vjp_sym[] = {
	GRAV_VJPSYM_ENTRY(2, 8, 64, true),
	GRAV_VJPSYM_ENTRY(2, 4, 64, true),
	GRAV_VJPSYM_ENTRY(4, 4, 128, true),
	GRAV_VJPSYM_ENTRY(2, 8, 64, false),
	GRAV_VJPSYM_ENTRY(2, 4, 64, false),
	GRAV_VJPSYM_ENTRY(4, 4, 128, false),
};

const VjpSymKernel* find_vjp_sym(int bpt, int threads, int jtile, bool fa)
{
	for (const VjpSymKernel& k : k_vjp_sym)
		if (k.bpt == bpt && k.threads == threads && k.jtile == jtile && k.fa == fa) return &k;
	return nullptr;
}

// Launch the unique-pair backward pair kernel (programmatic dependent; it waits with
// grid_dep_wait before it reads); fa: recompute the accelerations (7 slot components)
// or not (4).  Returns cudaErrorInvalidValue for a shape that is not compiled.
// Raise the kernel's dynamic shared-memory limit to its launch size (static plus dynamic
// above 48 KB needs the opt-in: the 4-rows-per-thread shapes), once per kernel and device.
static cudaError_t ensure_vjp_smem(const VjpSymKernel* k)
{
	static std::mutex mu;
	static std::set<std::pair<int, const void*>> done;
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	std::lock_guard<std::mutex> lock(mu);
	if (done.count({dev, k->fn})) return cudaSuccess;
	e = cudaFuncSetAttribute(k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, k->smem);
	if (e == cudaSuccess) done.insert({dev, k->fn});
	return e;
}

cudaError_t launch_vjp_sym(const grav_batch& b, const float4* upos, bool fa, cudaStream_t st)
{
	const VjpSymKernel* k = find_vjp_sym(b.tile.bpt, b.tile.threads, b.tile.jtile, fa);
	if (!k) return cudaErrorInvalidValue;
	cudaError_t e = ensure_vjp_smem(k);
	if (e != cudaSuccess) return e;
	grav_batch copy = b;
	void* args[] = {&copy, &upos};
	return launch_dependent(k->fn, b.tile.grid, k->threads, k->smem, st, args);
}

// Resident CTAs per SM: the smaller of the two variants' (the plan's grid serves both).
int vjp_sym_occupancy(int bpt, int threads, int jtile, int* ctas_per_sm)
{
	int best = -1;
	for (const bool fa : {true, false}) {
		const VjpSymKernel* k = find_vjp_sym(bpt, threads, jtile, fa);
		if (!k) return 0;
		int occ = 0;
		if (ensure_vjp_smem(k) != cudaSuccess ||
			cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k->fn, k->threads, k->smem) !=
				cudaSuccess)
			return -1;
		best = best < 0 ? occ : min(best, occ);
	}
	*ctas_per_sm = best;
	return 1;
}

}  // namespace grav
