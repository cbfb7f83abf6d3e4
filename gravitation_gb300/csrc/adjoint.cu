// adjoint.cu -- discrete adjoint (reverse-mode gradient) of the step, for gradients of
// a loss on the final state with respect to initial positions, velocities and masses.
//
// Forward step k (symplectic Euler, _base_.py:58-62):
//     a_k = A(r_k),  v_{k+1} = v_k + T a_k,  r_{k+1} = r_k + T v_{k+1}
//     A_i(r) = sum_{j!=i} Gm_j f(r_j - r_i),  f(d) = d/|d|^3
// Backward step k, given gr = dL/dr_{k+1}, gv = dL/dv_{k+1}:
//     u   = gv + T gr                         (dL/dv_{k+1} through both uses)
//     gr <- gr + T h_k,   h_k = J_A(r_k)^T u
//     gv <- u
//     gGm_j <- gGm_j + T sum_{i!=j} u_i . f(r_j - r_i)  = gGm_j - T g_j
// with, per ordered pair (k, j), d = r_j - r_k and Jf(d) = I/|d|^3 - 3 d d^T/|d|^5,
//     h_k = sum_j Jf(d) (Gm_k u_j - Gm_j u_k)
//         = Gm_k sum_j u_j/|d|^3 - u_k sum_j Gm_j/|d|^3 - 3 sum_j (Gm_k d.u_j - Gm_j d.u_k) d/|d|^5
//     g_k = sum_j u_j . d / |d|^3
// Zero separations (the self pair, coincident bodies) are excluded exactly (the
// reciprocal distance is selected to 0), so no large self terms enter the sums.
//
// The state needed by step k is not stored: the backward sweep reverses the forward
// update in FP64,  r_k = r_{k+1} - T v_{k+1},  v_k = v_{k+1} - T a_k.  a_k is either
// the forward's own FP64 acceleration of that step, kept by the caller (grav_adjoint
// a_in: what stage 2 wrote with GRAV_S2_WRITE_A), or recomputed as A(r_k) (stage 1)
// inside the same pair kernel as h and g (a_in NULL).  The caller resets the reversed
// state to the stored FP64 checkpoint at the start of every checkpoint segment, so
// rounding in the reversal never accumulates over more than one segment.
//
// Pair kernel: persistent stage-1 work list (pairs_skeleton.cuh), j-tiles of FP32
// positions (x, y, z, Gm) and FP32 u, FP32 tile partials folded into compensated
// (TwoSum) FP32 sums, so no FP64 arithmetic runs in the pair loop; 7 outputs
// per body (a, h, g) in the partial slots, as FP32 (hi, lo) pairs, or 4 (h, g) when
// the caller keeps the accelerations.  Adjoint stage 2 (1 or 8 lanes per padded row)
// sums the slots and applies the updates above in FP64, then prepares the FP32
// positions r_{k-1} and u for the next backward step.
#include <algorithm>

#include "pairs_skeleton.cuh"

namespace grav {

int record_error(int code, const char* msg);
// the unique-pair backward pair kernel (adjoint_sym.cu)
cudaError_t launch_vjp_sym(const grav_batch& b, const float4* upos, bool fa, cudaStream_t st);
int vjp_sym_occupancy(int bpt, int threads, int jtile, int* ctas_per_sm);

// FA_: recompute the accelerations (slot components a, h, g) or not (h, g)
template <int B_, int T_, int J_, bool FA_>
struct VjpOp {
	static constexpr bool FA = FA_;
	static constexpr int B = B_, T = T_, J = J_, NP = 2, NC = FA ? 7 : 4;
	static constexpr int H0 = FA ? 3 : 0, G0 = H0 + 3;
	using Elem = float4;
	const float4* pos;
	const float4* upos;
	float xi[B], yi[B], zi[B], gmi[B], uxi[B], uyi[B], uzi[B];
	float fa[3][B], fp[3][B], fq[3][B], fs[B], fg[B];
	// compensated (TwoSum) running sums: high and low FP32 parts
	float ah[3][B], al[3][B], hh[3][B], hl[3][B], gh[B], gl[B];

	__device__ const Elem* jsrc(int a) const { return a == 0 ? pos : upos; }

	__device__ void begin(int64_t ibase, int tid)
	{
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const float4 p = pos[ibase + tid + k * T];
			const float4 q = upos[ibase + tid + k * T];
			xi[k] = p.x;
			yi[k] = p.y;
			zi[k] = p.z;
			gmi[k] = p.w;
			uxi[k] = q.x;
			uyi[k] = q.y;
			uzi[k] = q.z;
#pragma unroll
			for (int c = 0; c < 3; ++c) {
				fa[c][k] = fp[c][k] = fq[c][k] = 0.f;
				ah[c][k] = al[c][k] = hh[c][k] = hl[c][k] = 0.f;
			}
			fs[k] = fg[k] = 0.f;
			gh[k] = gl[k] = 0.f;
		}
	}

	__device__ void tile(const Elem* const* s)
	{
		const float4* sp = s[0];
		const float4* su = s[1];
#pragma unroll 2
		for (int j = 0; j < J; ++j) {
			const float4 pj = sp[j];
			const float4 uj = su[j];
#pragma unroll
			for (int k = 0; k < B; ++k) {
				const float dx = pj.x - xi[k], dy = pj.y - yi[k], dz = pj.z - zi[k];
				const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
				const float inv = (r2 > 0.f) ? rsqrt_sfu(r2) : 0.f;
				const float inv2 = inv * inv;
				const float inv3 = inv2 * inv;
				const float inv5 = inv3 * inv2;  // the -3 of Jf is applied at the fold
				const float c = pj.w * inv3;  // Gm_j / r^3
				if constexpr (FA) {
					fa[0][k] = fmaf(c, dx, fa[0][k]);
					fa[1][k] = fmaf(c, dy, fa[1][k]);
					fa[2][k] = fmaf(c, dz, fa[2][k]);
				}
				fs[k] += c;
				fp[0][k] = fmaf(uj.x, inv3, fp[0][k]);
				fp[1][k] = fmaf(uj.y, inv3, fp[1][k]);
				fp[2][k] = fmaf(uj.z, inv3, fp[2][k]);
				const float duj = fmaf(dz, uj.z, fmaf(dy, uj.y, dx * uj.x));
				const float duk = fmaf(dz, uzi[k], fmaf(dy, uyi[k], dx * uxi[k]));
				const float dw = fmaf(gmi[k], duj, -pj.w * duk);
				const float t = dw * inv5;
				fq[0][k] = fmaf(t, dx, fq[0][k]);
				fq[1][k] = fmaf(t, dy, fq[1][k]);
				fq[2][k] = fmaf(t, dz, fq[2][k]);
				fg[k] = fmaf(duj, inv3, fg[k]);
			}
		}
		// fold the tile's FP32 partials into compensated FP32 (TwoSum) sums
#pragma unroll
		for (int k = 0; k < B; ++k) {
#pragma unroll
			for (int c3 = 0; c3 < 3; ++c3) {
				if constexpr (FA) two_sum_acc(ah[c3][k], al[c3][k], fa[c3][k]);
				fa[c3][k] = 0.f;
			}
			const float ui[3] = {uxi[k], uyi[k], uzi[k]};
#pragma unroll
			for (int c3 = 0; c3 < 3; ++c3) {
				// h = Gm_k P - u_k S - 3 Q
				const float ht = fmaf(gmi[k], fp[c3][k], fmaf(-ui[c3], fs[k], -3.f * fq[c3][k]));
				two_sum_acc(hh[c3][k], hl[c3][k], ht);
				fp[c3][k] = fq[c3][k] = 0.f;
			}
			two_sum_acc(gh[k], gl[k], fg[k]);
			fs[k] = fg[k] = 0.f;
		}
	}

	// the compensated sums go out as FP32 (hi, lo) pairs, one 8-byte slot entry each, with
	// no FP64 arithmetic; the adjoint stage 2 adds them in FP32 by TwoSum
	__device__ void store(double* out, int tid)
	{
		constexpr int IT = B * T;
		float2* out2 = reinterpret_cast<float2*>(out);
#pragma unroll
		for (int k = 0; k < B; ++k) {
			const int i = tid + k * T;
#pragma unroll
			for (int c3 = 0; c3 < 3; ++c3) {
				if constexpr (FA) out2[c3 * IT + i] = make_float2(ah[c3][k], al[c3][k]);
				out2[(H0 + c3) * IT + i] = make_float2(hh[c3][k], hl[c3][k]);
			}
			out2[G0 * IT + i] = make_float2(gh[k], gl[k]);
		}
	}
};

template <int B, int T, int J, bool FA>
__global__ void __launch_bounds__(T) vjp_kernel(const grav_batch b, const float4* upos)
{
	VjpOp<B, T, J, FA> op;
	op.pos = static_cast<const float4*>(b.pos);
	op.upos = upos;
	run_pairs(b, op);
}

struct __align__(32) arow4 {
	double x, y, z, w;
};

// flags of the adjoint stage 2
#define ADJ_STEP 1     // apply one backward step from the pair kernel's sums
#define ADJ_PREPARE 2  // write FP32 r_{k-1} = r - T v and u = gv + T gr for the pair kernel

// Lanes per row, as in stage2.cu: for small batches the row's slots are split over
// ATPR adjacent lanes of a warp (lane p takes slots p, p + ATPR, ...) and combined by a
// butterfly, which gives every lane the same bits; lane 0 then applies the row's
// update.  Large batches use one lane per row.
constexpr int AS2_THREADS = 128;
constexpr int ADJ_SPLIT_ROWS_MAX = 16384;  // ATPR = 8 up to this many padded rows, else 1

// NC: components per slot entry, 7 (a, h, g) or 4 (h, g: the accelerations come from
// a_in, the forward's own a_k rows).  With NC = 7 and a_in given, a_in is used.
template <int ATPR, int NC>
__global__ void __launch_bounds__(AS2_THREADS) adjoint_stage2_kernel(const grav_batch b,
	double* gr, double* gv, double* ggm, float4* upos, const double* a_in, const int flags)
{
	static_assert(ATPR > 0 && ATPR <= 16 && (ATPR & (ATPR - 1)) == 0 && AS2_THREADS % 32 == 0,
		"a row's lanes must sit in one warp");
	static_assert(NC == 7 || NC == 4, "slot components");
	constexpr int H0 = NC - 4, G0 = NC - 1;
	const int64_t gthread = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	const int64_t g = gthread / ATPR;  // padded row; the ATPR lanes of a row share a warp
	const int p = static_cast<int>(gthread % ATPR);
	const unsigned gmask = ((1u << ATPR) - 1) << ((threadIdx.x & 31) & ~(ATPR - 1));
	if (g >= b.n_pad_total) return;  // the whole lane group
	const int IT = b.tile.bpt * b.tile.threads;
	const int64_t seg = g / IT;
	const int li = static_cast<int>(g - seg * IT);
	const grav_seg_desc S = b.seg[seg];
	const grav_univ_desc U = b.univ[S.u];
	const int il = S.il0 + li;
	// slots, state, gradients and positions belong to the kernels before this one
	grid_dep_wait();
	float4* pos = static_cast<float4*>(b.pos);
	if (il >= U.n) {  // the whole lane group
		if (p == 0) {
			pos[g] = make_float4(0.f, 0.f, 0.f, 0.f);
			upos[g] = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		return;
	}
	const int64_t row = U.body_off + il;
	const double T = U.T;
	// Split rows (ATPR >= 4) spread the row's FP64 work over its lanes: lane c < 3 takes
	// component c of r, v, gr, gv (and of a and h), lane 3 the mass terms.  GB300 issues an
	// FP64 warp instruction at the same cost whatever the number of active lanes, so this
	// cuts a warp's FP64 instructions about 3x against one lane doing the whole row.  With
	// one lane per row (ATPR = 1) every lane already holds a row of its own.
	constexpr bool SPLIT = ATPR >= 4;
	arow4* rr = reinterpret_cast<arow4*>(b.r);
	arow4* vv = reinterpret_cast<arow4*>(b.v);
	arow4* grr = reinterpret_cast<arow4*>(gr);
	arow4* gvv = reinterpret_cast<arow4*>(gv);
	double* rd = static_cast<double*>(b.r);
	double* vd = static_cast<double*>(b.v);
	const int64_t e = 4 * row + (p < 3 ? p : 3);  // this lane's component (SPLIT)
	// the row's state goes out before the slot loads
	arow4 r = {0.0, 0.0, 0.0, 0.0}, v = r, a_gr = r, a_gv = r, acc = r;
	double rc = 0.0, vc = 0.0, grc = 0.0, gvc = 0.0, ac = 0.0;
	double gm_acc = 0.0;
	if (SPLIT) {
		if (p < 4) {
			rc = rd[e];  // x, y, z or G*m
			if (p < 3) {
				vc = vd[e];
				grc = gr[e];
				gvc = gv[e];
				if ((flags & ADJ_STEP) && a_in) ac = __ldcs(a_in + e);  // read once: evict-first
			} else if (flags & ADJ_STEP) {
				gm_acc = ggm[row];
			}
		}
	} else if (p == 0) {
		r = rr[row];
		v = vv[row];
		a_gr = grr[row];
		a_gv = gvv[row];
		if (flags & ADJ_STEP) gm_acc = ggm[row];
		if ((flags & ADJ_STEP) && a_in) {  // read once: evict-first
			const double2* ai = reinterpret_cast<const double2*>(a_in) + 2 * row;
			const double2 axy = __ldcs(ai), az = __ldcs(ai + 1);
			acc = arow4{axy.x, axy.y, az.x, 0.0};
		}
	}

	float h[NC], l[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) h[c] = l[c] = 0.f;
	if (flags & ADJ_STEP) {
		// slots p, p + ATPR, ... hold FP32 (hi, lo) pairs; they are added in order into
		// compensated FP32 sums (hi by TwoSum, lo and the errors into l), each round
		// issuing all its loads first, and combined across the lanes by a TwoSum butterfly
		// that leaves every lane with the same bits: no FP64 arithmetic per slot (GB300
		// runs FP64 at ~1/64 of the FP32 rate)
		constexpr int SLOT_BATCH = NC == 4 ? 6 : 4;
		const int64_t stride = NC * static_cast<int64_t>(IT);  // 8-byte entries per slot
		// unique-pair plans: the last (row block index) slots of a segment are column
		// slots holding FP32 values in their first half (adjoint_sym.cu)
		const int nrow = b.mode == GRAV_MODE_FP32U ? S.nslots - S.il0 / IT : S.nslots;
		const float2* part =
			reinterpret_cast<const float2*>(b.part + static_cast<int64_t>(S.slot_base) * stride) + li;
		const float* cpart =
			reinterpret_cast<const float*>(b.part + static_cast<int64_t>(S.slot_base) * stride) + li;
		// row and column slots share one index space and one round of loads per batch
		// (slots past the end read as 0, added exactly)
		for (int k = p; k < S.nslots; k += SLOT_BATCH * ATPR) {
			float2 q[SLOT_BATCH][NC];
#pragma unroll
			for (int j = 0; j < SLOT_BATCH; ++j) {
				const int kk = k + j * ATPR;
				if (kk < nrow) {
#pragma unroll
					for (int c = 0; c < NC; ++c) q[j][c] = __ldg(part + kk * stride + c * IT);
				} else if (kk < S.nslots) {
#pragma unroll
					for (int c = 0; c < NC; ++c)
						q[j][c] = make_float2(__ldg(cpart + kk * 2 * stride + c * IT), 0.f);
				} else {
#pragma unroll
					for (int c = 0; c < NC; ++c) q[j][c] = make_float2(0.f, 0.f);
				}
			}
#pragma unroll
			for (int j = 0; j < SLOT_BATCH; ++j)
#pragma unroll
				for (int c = 0; c < NC; ++c) {
					two_sum_acc(h[c], l[c], q[j][c].x);
					l[c] += q[j][c].y;
				}
		}
#pragma unroll
		for (int c = 0; c < NC; ++c) group_sum_pair<ATPR>(h[c], l[c], gmask);
	}

	if (SPLIT) {
		if (p >= 4) return;
		float* posf = reinterpret_cast<float*>(pos) + 4 * g + p;
		float* uposf = reinterpret_cast<float*>(upos) + 4 * g + p;
		if (p == 3) {  // mass terms
			if (flags & ADJ_STEP)
				ggm[row] = gm_acc - T * (static_cast<double>(h[G0]) + static_cast<double>(l[G0]));
			if (flags & ADJ_PREPARE) {
				*posf = __double2float_rn(rc);
				*uposf = 0.f;
			}
			return;
		}
		if (flags & ADJ_STEP) {
			// this lane's component of a (recomputed, NC = 7 without a_in) and of h
			const int ca = p, ch = H0 + p;
			const float a_h = ca == 0 ? h[0] : (ca == 1 ? h[1] : h[2]);
			const float a_l = ca == 0 ? l[0] : (ca == 1 ? l[1] : l[2]);
			const float h_h = ch == H0 ? h[H0] : (ch == H0 + 1 ? h[H0 + 1] : h[H0 + 2]);
			const float h_l = ch == H0 ? l[H0] : (ch == H0 + 1 ? l[H0 + 1] : l[H0 + 2]);
			if (NC == 7 && !a_in) ac = static_cast<double>(a_h) + static_cast<double>(a_l);
			const double hc = static_cast<double>(h_h) + static_cast<double>(h_l);
			// reverse the forward update: r_k = r_{k+1} - T v_{k+1}; v_k = v_{k+1} - T a_k
			rc = __dsub_rn(rc, __dmul_rn(vc, T));
			vc = __dsub_rn(vc, __dmul_rn(ac, T));
			// gradients
			const double uc = gvc + T * grc;
			grc += T * hc;
			gvc = uc;
			rd[e] = rc;
			vd[e] = vc;
			gr[e] = grc;
			gv[e] = gvc;
		}
		if (flags & ADJ_PREPARE) {
			// position of the next backward step and the u it contracts with
			*posf = __double2float_rn(__dsub_rn(rc, __dmul_rn(vc, T)));
			*uposf = __double2float_rn(gvc + T * grc);
		}
		return;
	}

	if (p != 0) return;
	double s[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) s[c] = static_cast<double>(h[c]) + static_cast<double>(l[c]);
	if (flags & ADJ_STEP) {
		// reverse the forward update: r_k = r_{k+1} - T v_{k+1}; v_k = v_{k+1} - T a_k
		if (NC == 7 && !a_in) acc = arow4{s[0], s[1], s[2], 0.0};
		r.x = __dsub_rn(r.x, __dmul_rn(v.x, T));
		r.y = __dsub_rn(r.y, __dmul_rn(v.y, T));
		r.z = __dsub_rn(r.z, __dmul_rn(v.z, T));
		v.x = __dsub_rn(v.x, __dmul_rn(acc.x, T));
		v.y = __dsub_rn(v.y, __dmul_rn(acc.y, T));
		v.z = __dsub_rn(v.z, __dmul_rn(acc.z, T));
		// gradients
		const double ux = a_gv.x + T * a_gr.x, uy = a_gv.y + T * a_gr.y, uz = a_gv.z + T * a_gr.z;
		a_gr.x += T * s[H0];
		a_gr.y += T * s[H0 + 1];
		a_gr.z += T * s[H0 + 2];
		a_gv.x = ux;
		a_gv.y = uy;
		a_gv.z = uz;
		ggm[row] = gm_acc - T * s[G0];
		rr[row] = r;
		vv[row] = v;
		grr[row] = a_gr;
		gvv[row] = a_gv;
	}
	if (flags & ADJ_PREPARE) {
		// position of the next backward step and the u it contracts with
		const double px = __dsub_rn(r.x, __dmul_rn(v.x, T));
		const double py = __dsub_rn(r.y, __dmul_rn(v.y, T));
		const double pz = __dsub_rn(r.z, __dmul_rn(v.z, T));
		pos[g] = make_float4(__double2float_rn(px), __double2float_rn(py), __double2float_rn(pz),
			__double2float_rn(r.w));
		upos[g] = make_float4(__double2float_rn(a_gv.x + T * a_gr.x),
			__double2float_rn(a_gv.y + T * a_gr.y), __double2float_rn(a_gv.z + T * a_gr.z), 0.f);
	}
}

// Adjoint stage 2 as a programmatic dependent of the kernel before it (it waits with
// grid_dep_wait); 8 lanes per padded row for small batches, else 1; nc slot components.
cudaError_t launch_adjoint_stage2(const grav_batch& b, const grav_adjoint& a, int flags, int nc,
	cudaStream_t st)
{
	grav_batch copy = b;
	double* gr = static_cast<double*>(a.gr);
	double* gv = static_cast<double*>(a.gv);
	double* ggm = static_cast<double*>(a.ggm);
	float4* upos = static_cast<float4*>(a.upos);
	const double* a_in = a.a_in;
	int f = flags;
	void* args[] = {&copy, &gr, &gv, &ggm, &upos, &a_in, &f};
	const int atpr = b.n_pad_total <= ADJ_SPLIT_ROWS_MAX ? 8 : 1;
	const unsigned blocks =
		static_cast<unsigned>((b.n_pad_total * atpr + AS2_THREADS - 1) / AS2_THREADS);
	const void* fn = nc == 4
		? (atpr == 8 ? reinterpret_cast<const void*>(&adjoint_stage2_kernel<8, 4>)
		             : reinterpret_cast<const void*>(&adjoint_stage2_kernel<1, 4>))
		: (atpr == 8 ? reinterpret_cast<const void*>(&adjoint_stage2_kernel<8, 7>)
		             : reinterpret_cast<const void*>(&adjoint_stage2_kernel<1, 7>));
	return launch_dependent(fn, blocks, AS2_THREADS, 0, st, args);
}

struct VjpKernel {
	int bpt, threads, jtile;
	bool fa;
	const void* fn;
	int smem;
};

#define GRAV_VJP_ENTRY(B, T, J, FA) \
	{B, T, J, FA, reinterpret_cast<const void*>(&vjp_kernel<B, T, J, FA>), \
		pairs_smem_bytes<VjpOp<B, T, J, FA>>()}

static const VjpKernel k_vjp[] = {
	GRAV_VJP_ENTRY(1, 128, 128, true),
	GRAV_VJP_ENTRY(2, 128, 128, true),
	GRAV_VJP_ENTRY(2, 256, 128, true),
	GRAV_VJP_ENTRY(4, 128, 128, true),
	GRAV_VJP_ENTRY(1, 128, 128, false),
	GRAV_VJP_ENTRY(2, 128, 128, false),
	GRAV_VJP_ENTRY(2, 256, 128, false),
	GRAV_VJP_ENTRY(4, 128, 128, false),
};

int vjp_table(const VjpKernel** out)
{
	*out = k_vjp;
	return static_cast<int>(sizeof(k_vjp) / sizeof(k_vjp[0]));
}

}  // namespace grav

namespace {

int check_adj(const grav_adjoint* a)
{
	using grav::record_error;
	if (!a || !a->b) return record_error(GRAV_E_ARG, "NULL adjoint or batch");
	const grav_batch* b = a->b;
	if (b->mode != GRAV_MODE_FP32 && b->mode != GRAV_MODE_FP32U)
		return record_error(GRAV_E_ARG, "the adjoint runs on an FP32 (all pairs, grav_plan) or "
			"FP32U (unique pairs, grav_plan_pairs) batch");
	if (!b->univ || !b->seg || !b->pos || !b->r || !b->v || !b->err)
		return record_error(GRAV_E_ARG, "NULL device pointer in grav_batch");
	if (!a->gr || !a->gv || !a->ggm || !a->upos || !a->part7)
		return record_error(GRAV_E_ARG, "NULL device pointer in grav_adjoint");
	const int64_t itile = static_cast<int64_t>(b->tile.bpt) * b->tile.threads;
	if (b->n_pad_total != static_cast<int64_t>(b->n_seg) * itile)
		return record_error(GRAV_E_ARG, "n_pad_total != n_seg * itile");
	return GRAV_OK;
}

}  // namespace

extern "C" int grav_adjoint_tile_supported(int mode, const grav_tile* t)
{
	if (!t) return 0;
	if (mode == GRAV_MODE_FP32U) {
		int occ = 0;
		return grav::vjp_sym_occupancy(t->bpt, t->threads, t->jtile, &occ) != 0 ? 1 : 0;
	}
	if (mode != GRAV_MODE_FP32) return 0;
	const grav::VjpKernel* tab = nullptr;
	const int n = grav::vjp_table(&tab);
	for (int i = 0; i < n; ++i)
		if (tab[i].bpt == t->bpt && tab[i].threads == t->threads && tab[i].jtile == t->jtile) return 1;
	return 0;
}

extern "C" int grav_adjoint_occupancy(int mode, const grav_tile* t, int32_t* ctas_per_sm)
{
	if (!t || !ctas_per_sm) return grav::record_error(GRAV_E_ARG, "NULL argument");
	if (mode == GRAV_MODE_FP32U) {
		int occ = 0;
		const int rc = grav::vjp_sym_occupancy(t->bpt, t->threads, t->jtile, &occ);
		if (rc == 0) return grav::record_error(GRAV_E_TILE, "tile shape has no unique-pair adjoint kernel");
		if (rc < 0) return grav::record_error(GRAV_E_CUDA, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
		*ctas_per_sm = occ;
		return GRAV_OK;
	}
	if (mode != GRAV_MODE_FP32) return grav::record_error(GRAV_E_ARG, "adjoint mode must be FP32 or FP32U");
	const grav::VjpKernel* tab = nullptr;
	const int n = grav::vjp_table(&tab);
	int best = -1;  // the smaller of the two variants' (the plan's grid serves both)
	for (int i = 0; i < n; ++i)
		if (tab[i].bpt == t->bpt && tab[i].threads == t->threads && tab[i].jtile == t->jtile) {
			int blocks = 0;
			cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, tab[i].fn,
				tab[i].threads, tab[i].smem);
			if (e != cudaSuccess) return grav::record_error(GRAV_E_CUDA, cudaGetErrorString(e));
			best = best < 0 ? blocks : std::min(best, blocks);
		}
	if (best < 0) return grav::record_error(GRAV_E_TILE, "tile shape has no adjoint kernel");
	*ctas_per_sm = best;
	return GRAV_OK;
}

extern "C" int grav_adjoint_prepare(const grav_adjoint* a, void* stream)
{
	int rc = check_adj(a);
	if (rc) return rc;
	const grav_batch& b = *a->b;
	if (b.n_pad_total == 0) return GRAV_OK;
	grav_batch copy = b;
	copy.part = a->part7;
	cudaError_t e = grav::launch_adjoint_stage2(copy, *a, ADJ_PREPARE, 7, static_cast<cudaStream_t>(stream));
	return e == cudaSuccess ? GRAV_OK : grav::record_error(GRAV_E_CUDA, cudaGetErrorString(e));
}

extern "C" int grav_adjoint_step(const grav_adjoint* a, void* stream)
{
	int rc = check_adj(a);
	if (rc) return rc;
	const grav_batch& b = *a->b;
	if (b.n_pad_total == 0) return GRAV_OK;
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	grav_batch copy = b;
	copy.part = a->part7;
	// with the forward's accelerations at hand the pair kernel forms only h and g
	const bool fa = a->a_in == nullptr;
	if (b.n_units > 0) {
		if (b.tile.grid <= 0 || b.tile.grid > b.n_units)
			return grav::record_error(GRAV_E_ARG, "tile.grid must be in [1, n_units]");
		const float4* up = static_cast<const float4*>(a->upos);
		if (b.mode == GRAV_MODE_FP32U) {
			const cudaError_t e = grav::launch_vjp_sym(copy, up, fa, st);
			if (e == cudaErrorInvalidValue)
				return grav::record_error(GRAV_E_TILE, "tile shape has no unique-pair adjoint kernel");
			if (e != cudaSuccess) return grav::record_error(GRAV_E_CUDA, cudaGetErrorString(e));
		} else {
			const grav::VjpKernel* tab = nullptr;
			const int n = grav::vjp_table(&tab);
			const grav::VjpKernel* k = nullptr;
			for (int i = 0; i < n; ++i)
				if (tab[i].bpt == b.tile.bpt && tab[i].threads == b.tile.threads &&
					tab[i].jtile == b.tile.jtile && tab[i].fa == fa)
					k = &tab[i];
			if (!k) return grav::record_error(GRAV_E_TILE, "tile shape has no adjoint kernel");
			void* args[] = {&copy, &up};
			const cudaError_t e = grav::launch_dependent(k->fn, b.tile.grid, k->threads, k->smem, st, args);
			if (e != cudaSuccess) return grav::record_error(GRAV_E_CUDA, cudaGetErrorString(e));
		}
	}
	cudaError_t e = grav::launch_adjoint_stage2(copy, *a, ADJ_STEP | ADJ_PREPARE, fa ? 7 : 4, st);
	return e == cudaSuccess ? GRAV_OK : grav::record_error(GRAV_E_CUDA, cudaGetErrorString(e));
}
