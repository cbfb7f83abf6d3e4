// scenario.cu -- seeded scenarios generated on the device into the packed FP64 state.
//
// Random numbers: Philox4x64-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
// as easy as 1, 2, 3", SC'11), keyed by {seed, stream} and counted by {body, block}, so
// each body's draws are independent of every other body and of the launch shape.  A
// uniform double is (word >> 11) * 2^-53.  Products and sums that decide bits are
// written with explicit round-to-nearest intrinsics (no FMA contraction), so a CPU
// restatement compiled without contraction reproduces the uniform-derived values
// bit for bit; values that pass through log/exp/sin/cos/expm1 agree to a few ulp.
//
// Scenarios (see grav_scenario in the header):
//   cube     r ~ U[-h, h]^3, v ~ N(0, sigma^2)^3 (Box-Muller), m ~ U[m_lo, m_hi]
//   plummer  one Plummer sphere, Aarseth, Henon & Wielen (1974); three launches:
//            masses (+ per-CTA sums of G*m), bodies (+ per-CTA sums of G*m*r, G*m*v),
//            shift of the centre of mass; every CTA adds the per-CTA sums in the same
//            fixed order, so the result does not depend on scheduling
//   galaxy   the reference's recipe (simulation.py:99-184) with the zero galaxy
//            rotations left out, scaled as add_object scales (_base_.py:114-117)
// All three write r = (x, y, z, G*m) and v = (vx, vy, vz, 0) rows; HBM-write bound.
#include <cmath>

#include "grav_device.cuh"

namespace grav {
int record_error(int code, const char* msg);
}

namespace {

constexpr uint64_t PHILOX_M0 = 0xD2E7470EE14C6C93ull;
constexpr uint64_t PHILOX_M1 = 0xCA5A826395121157ull;
constexpr uint64_t PHILOX_W0 = 0x9E3779B97F4A7C15ull;  // golden ratio
constexpr uint64_t PHILOX_W1 = 0xBB67AE8584CAA73Bull;  // sqrt(3) - 1
constexpr double TWO_PI = 6.283185307179586;
constexpr double PI = 3.141592653589793;
constexpr double HALF_PI = 1.5707963267948966;
constexpr double Q_FALLBACK = 0.4714045207910317;  // sqrt(2/9): the maximum of g(q)
constexpr int THREADS = 256;
constexpr int MAX_CTAS = 1024;
constexpr int REJECT_BLOCKS = 32;  // 64 trials; P(all rejected) ~ 0.57^64 ~ 2e-16
constexpr int PART_STRIDE = 8;     // doubles per CTA in the Plummer scratch

struct __align__(32) row4 {
	double x, y, z, w;
};

struct ScenArgs {
	uint64_t seed, stream;
	double G;
	double p[10];
	double ln_lo, ln_hi;  // Plummer: log(m_lo), log(m_hi), formed on the host
};

// Philox4x64 with 10 rounds on the counter {c0, c1, 0, 0}.
__device__ __forceinline__ void philox(uint64_t c0, uint64_t c1, uint64_t k0, uint64_t k1,
	uint64_t out[4])
{
	uint64_t x0 = c0, x1 = c1, x2 = 0, x3 = 0;
#pragma unroll
	for (int round = 0; round < 10; ++round) {
		const uint64_t lo0 = PHILOX_M0 * x0, hi0 = __umul64hi(PHILOX_M0, x0);
		const uint64_t lo1 = PHILOX_M1 * x2, hi1 = __umul64hi(PHILOX_M1, x2);
		x0 = hi1 ^ x1 ^ k0;
		x1 = lo1;
		x2 = hi0 ^ x3 ^ k1;
		x3 = lo0;
		k0 += PHILOX_W0;
		k1 += PHILOX_W1;
	}
	out[0] = x0;
	out[1] = x1;
	out[2] = x2;
	out[3] = x3;
}

__device__ __forceinline__ double u01(uint64_t w)
{
	return __dmul_rn(static_cast<double>(w >> 11), 0x1.0p-53);
}

// lo + (hi - lo) * u, each operation rounded
__device__ __forceinline__ double lin(double lo, double hi, double u)
{
	return __dadd_rn(lo, __dmul_rn(__dsub_rn(hi, lo), u));
}

// A point at distance `rad` in the direction given by two uniforms:
// z = (1 - 2 uc) rad, phi = 2 pi up, rho = sqrt(max(rad^2 - z^2, 0)).
__device__ __forceinline__ void isotropic(double uc, double up, double rad, double& x,
	double& y, double& z)
{
	z = __dmul_rn(__dsub_rn(1.0, __dmul_rn(2.0, uc)), rad);
	const double phi = __dmul_rn(TWO_PI, up);
	const double rho = sqrt(fmax(__dsub_rn(__dmul_rn(rad, rad), __dmul_rn(z, z)), 0.0));
	x = __dmul_rn(rho, cos(phi));
	y = __dmul_rn(rho, sin(phi));
}

// Block sum in a fixed order (per-thread sums, then a fixed shared-memory tree).
template <int K>
__device__ __forceinline__ void block_sum(double (&acc)[K], double* out)
{
	__shared__ double sh[K][THREADS];
	for (int k = 0; k < K; ++k) sh[k][threadIdx.x] = acc[k];
	__syncthreads();
	for (int s = THREADS / 2; s > 0; s >>= 1) {
		if (threadIdx.x < s)
			for (int k = 0; k < K; ++k)
				sh[k][threadIdx.x] = __dadd_rn(sh[k][threadIdx.x], sh[k][threadIdx.x + s]);
		__syncthreads();
	}
	if (threadIdx.x == 0)
		for (int k = 0; k < K; ++k) out[k] = sh[k][0];
}

// Sum of column `k` of the per-CTA scratch over nb CTAs, the same bits in every CTA and
// lane: lane l adds rows l, l+32, ... in order, then a butterfly (each pair's sum is
// formed from the same two operands on both sides, and IEEE addition commutes).
__device__ __forceinline__ double sum_parts(const double* part, int nb, int k)
{
	const int lane = threadIdx.x & 31;
	double s = 0.0;
	for (int b = lane; b < nb; b += 32) s = __dadd_rn(s, part[b * PART_STRIDE + k]);
	for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
	return s;
}

__global__ void __launch_bounds__(THREADS) cube_kernel(row4* __restrict__ r, row4* __restrict__ v,
	const int64_t n, const ScenArgs a)
{
	const double h = a.p[0], sigma = a.p[1];
	for (int64_t i = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; i < n;
		 i += static_cast<int64_t>(gridDim.x) * THREADS) {
		uint64_t w[4], u[4];
		philox(static_cast<uint64_t>(i), 0, a.seed, a.stream, w);
		philox(static_cast<uint64_t>(i), 1, a.seed, a.stream, u);
		row4 R, V;
		R.x = lin(-h, h, u01(w[0]));
		R.y = lin(-h, h, u01(w[1]));
		R.z = lin(-h, h, u01(w[2]));
		R.w = __dmul_rn(a.G, lin(a.p[2], a.p[3], u01(w[3])));
		// Box-Muller: rad = sqrt(-2 log(1 - u)), angle = 2 pi u'
		const double rad0 = sqrt(__dmul_rn(-2.0, log(__dsub_rn(1.0, u01(u[0])))));
		const double th0 = __dmul_rn(TWO_PI, u01(u[1]));
		const double rad1 = sqrt(__dmul_rn(-2.0, log(__dsub_rn(1.0, u01(u[2])))));
		const double th1 = __dmul_rn(TWO_PI, u01(u[3]));
		V.x = __dmul_rn(sigma, __dmul_rn(rad0, cos(th0)));
		V.y = __dmul_rn(sigma, __dmul_rn(rad0, sin(th0)));
		V.z = __dmul_rn(sigma, __dmul_rn(rad1, cos(th1)));
		V.w = 0.0;
		r[i] = R;
		v[i] = V;
	}
}

__global__ void __launch_bounds__(THREADS) plummer_mass_kernel(row4* __restrict__ r,
	const int64_t n, const ScenArgs a, double* __restrict__ part)
{
	double acc[1] = {0.0};
	for (int64_t i = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; i < n;
		 i += static_cast<int64_t>(gridDim.x) * THREADS) {
		uint64_t w[4];
		philox(static_cast<uint64_t>(i), 0, a.seed, a.stream, w);
		const double gm = __dmul_rn(a.G, exp(lin(a.ln_lo, a.ln_hi, u01(w[0]))));
		r[i] = row4{0.0, 0.0, 0.0, gm};
		acc[0] = __dadd_rn(acc[0], gm);
	}
	block_sum<1>(acc, part + blockIdx.x * PART_STRIDE);
}

__global__ void __launch_bounds__(THREADS) plummer_body_kernel(row4* __restrict__ r,
	row4* __restrict__ v, const int64_t n, const ScenArgs a, double* __restrict__ part)
{
	const double scale = a.p[0];
	const double gm_tot = sum_parts(part, gridDim.x, 0);
	// escape speed at the centre, sqrt(2 G M / a)
	const double vesc0 = sqrt(__ddiv_rn(__dmul_rn(2.0, gm_tot), scale));
	double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
	for (int64_t i = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; i < n;
		 i += static_cast<int64_t>(gridDim.x) * THREADS) {
		uint64_t w[4], d[4];
		philox(static_cast<uint64_t>(i), 0, a.seed, a.stream, w);
		philox(static_cast<uint64_t>(i), 1, a.seed, a.stream, d);
		// radius from M(r)/M = r^3/(r^2+a^2)^(3/2) = X, cut at X = 0.999:
		// r = a / sqrt(X^(-2/3) - 1), with X^(-2/3) - 1 = expm1(-2/3 log X)
		const double X = lin(1e-10, 0.999, u01(w[1]));
		const double rad = __ddiv_rn(scale, sqrt(expm1(__dmul_rn(-2.0 / 3.0, log(X)))));
		row4 R, V;
		isotropic(u01(w[2]), u01(w[3]), rad, R.x, R.y, R.z);
		// speed = q v_esc(r), q from g(q) = q^2 (1 - q^2)^(7/2) < 0.1 by rejection
		double q = Q_FALLBACK;
		bool found = false;
		for (int blk = 2; blk < 2 + REJECT_BLOCKS && !found; ++blk) {
			uint64_t t[4];
			philox(static_cast<uint64_t>(i), static_cast<uint64_t>(blk), a.seed, a.stream, t);
			for (int k = 0; k < 4 && !found; k += 2) {
				const double x4 = u01(t[k]), x5 = u01(t[k + 1]);
				const double x2 = __dmul_rn(x4, x4);
				const double y = __dsub_rn(1.0, x2);
				const double g = __dmul_rn(__dmul_rn(x2, __dmul_rn(__dmul_rn(y, y), y)), sqrt(y));
				if (__dmul_rn(0.1, x5) < g) {
					q = x4;
					found = true;
				}
			}
		}
		// v_esc(r) = v_esc(0) (1 + (r/a)^2)^(-1/4)
		const double xr = __ddiv_rn(rad, scale);
		const double ve = __ddiv_rn(vesc0, sqrt(sqrt(__dadd_rn(1.0, __dmul_rn(xr, xr)))));
		isotropic(u01(d[0]), u01(d[1]), __dmul_rn(q, ve), V.x, V.y, V.z);
		R.w = r[i].w;
		V.w = 0.0;
		r[i] = R;
		v[i] = V;
		acc[0] = __dadd_rn(acc[0], __dmul_rn(R.w, R.x));
		acc[1] = __dadd_rn(acc[1], __dmul_rn(R.w, R.y));
		acc[2] = __dadd_rn(acc[2], __dmul_rn(R.w, R.z));
		acc[3] = __dadd_rn(acc[3], __dmul_rn(R.w, V.x));
		acc[4] = __dadd_rn(acc[4], __dmul_rn(R.w, V.y));
		acc[5] = __dadd_rn(acc[5], __dmul_rn(R.w, V.z));
	}
	block_sum<6>(acc, part + blockIdx.x * PART_STRIDE + 1);
}

__global__ void __launch_bounds__(THREADS) plummer_shift_kernel(row4* __restrict__ r,
	row4* __restrict__ v, const int64_t n, const ScenArgs a, const double* __restrict__ part)
{
	const double gm_tot = sum_parts(part, gridDim.x, 0);
	double c[6];
	for (int k = 0; k < 6; ++k) c[k] = __ddiv_rn(sum_parts(part, gridDim.x, 1 + k), gm_tot);
	for (int64_t i = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; i < n;
		 i += static_cast<int64_t>(gridDim.x) * THREADS) {
		row4 R = r[i], V = v[i];
		R.x = __dadd_rn(__dsub_rn(R.x, c[0]), a.p[3]);
		R.y = __dadd_rn(__dsub_rn(R.y, c[1]), a.p[4]);
		R.z = __dadd_rn(__dsub_rn(R.z, c[2]), a.p[5]);
		V.x = __dadd_rn(__dsub_rn(V.x, c[3]), a.p[6]);
		V.y = __dadd_rn(__dsub_rn(V.y, c[4]), a.p[7]);
		V.z = __dadd_rn(__dsub_rn(V.z, c[5]), a.p[8]);
		r[i] = R;
		v[i] = V;
	}
}

__global__ void __launch_bounds__(THREADS) galaxy_kernel(row4* __restrict__ r, row4* __restrict__ v,
	const int64_t n, const ScenArgs a)
{
	const double radius = a.p[0], m_hole = a.p[1], m_star = a.p[2], sr = a.p[3], sm = a.p[4];
	const int64_t stars = n - 1;
	const int64_t n_disc = stars * 4 / 5;
	const double span = __dmul_rn(__dadd_rn(4.5, 0.1), radius);
	const double gm_hole = __dmul_rn(a.G, m_hole);
	for (int64_t i = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; i < n;
		 i += static_cast<int64_t>(gridDim.x) * THREADS) {
		if (i == 0) {
			r[0] = row4{0.0, 0.0, 0.0, __dmul_rn(a.G, __dmul_rn(m_hole, sm))};
			v[0] = row4{0.0, 0.0, 0.0, 0.0};
			continue;
		}
		uint64_t w[4];
		philox(static_cast<uint64_t>(i), 0, a.seed, a.stream, w);
		const double alpha = __dmul_rn(__dmul_rn(u01(w[0]), 2.0), PI);
		double x, y, z;
		if (i - 1 < n_disc) {
			const double r_abs = __dmul_rn(__dadd_rn(__dmul_rn(u01(w[1]), 4.5), 0.1), radius);
			x = __dmul_rn(r_abs, cos(alpha));
			y = __dmul_rn(r_abs, sin(alpha));
			z = __ddiv_rn(__dmul_rn(__dmul_rn(__dsub_rn(__dmul_rn(0.5, u01(w[2])), 0.25), radius),
							  __dsub_rn(span, r_abs)),
				span);
		} else {
			const double r_abs = __dmul_rn(__dadd_rn(__dmul_rn(u01(w[1]), 0.75), 0.1), radius);
			const double beta = __dmul_rn(PI, __dsub_rn(u01(w[2]), 0.5));
			x = __dmul_rn(__dmul_rn(r_abs, cos(alpha)), cos(beta));
			y = __dmul_rn(__dmul_rn(r_abs, sin(alpha)), cos(beta));
			z = __dmul_rn(r_abs, sin(beta));
		}
		const double dist = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
		const double v_abs = sqrt(__ddiv_rn(gm_hole, dist));
		const double va = __dsub_rn(alpha, HALF_PI);
		r[i] = row4{__dmul_rn(x, sr), __dmul_rn(y, sr), __dmul_rn(z, sr),
			__dmul_rn(a.G, __dmul_rn(m_star, sm))};
		v[i] = row4{__dmul_rn(__dmul_rn(v_abs, cos(va)), sr), __dmul_rn(__dmul_rn(v_abs, sin(va)), sr),
			0.0, 0.0};
	}
}

int ctas_for(int64_t n)
{
	const int64_t b = (n + THREADS - 1) / THREADS;
	return static_cast<int>(b < 1 ? 1 : (b > MAX_CTAS ? MAX_CTAS : b));
}

bool finite_all(const double* p, int k)
{
	for (int i = 0; i < k; ++i)
		if (!std::isfinite(p[i])) return false;
	return true;
}

}  // namespace

extern "C" {

int64_t grav_scenario_scratch_bytes(const grav_scenario* s, int64_t n)
{
	if (!s || n < 0) return grav::record_error(GRAV_E_ARG, "NULL scenario or n < 0");
	if (s->kind != GRAV_SCEN_PLUMMER) return 0;
	return static_cast<int64_t>(ctas_for(n)) * PART_STRIDE * sizeof(double);
}

int grav_scenario_generate(const grav_scenario* s, double* r, double* v, int64_t n,
	void* scratch, void* stream)
{
	using grav::record_error;
	if (!s) return record_error(GRAV_E_ARG, "NULL scenario");
	if (n < 0 || n > (int64_t(1) << 40)) return record_error(GRAV_E_SIZE, "n out of range");
	if (n == 0) return GRAV_OK;
	if (!r || !v) return record_error(GRAV_E_ARG, "NULL r or v");
	if ((reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(v)) & 31)
		return record_error(GRAV_E_ARG, "r and v must be 32-byte aligned");
	if (!std::isfinite(s->G) || s->G < 0.0 || !finite_all(s->p, 10))
		return record_error(GRAV_E_ARG, "G and the scenario parameters must be finite, G >= 0");
	ScenArgs a;
	a.seed = s->seed;
	a.stream = s->stream;
	a.G = s->G;
	for (int k = 0; k < 10; ++k) a.p[k] = s->p[k];
	a.ln_lo = a.ln_hi = 0.0;
	const int ctas = ctas_for(n);
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	row4* R = reinterpret_cast<row4*>(r);
	row4* V = reinterpret_cast<row4*>(v);
	switch (s->kind) {
	case GRAV_SCEN_UNIFORM_CUBE:
		if (!(a.p[0] >= 0.0 && a.p[1] >= 0.0 && a.p[2] >= 0.0 && a.p[3] >= a.p[2]))
			return record_error(GRAV_E_ARG, "uniform cube: need half >= 0, v_sigma >= 0, "
				"0 <= m_lo <= m_hi");
		cube_kernel<<<ctas, THREADS, 0, st>>>(R, V, n, a);
		break;
	case GRAV_SCEN_PLUMMER: {
		if (!(a.p[0] > 0.0 && a.p[1] > 0.0 && a.p[2] >= a.p[1]))
			return record_error(GRAV_E_ARG, "Plummer: need a > 0 and 0 < m_lo <= m_hi");
		if (!(a.G > 0.0)) return record_error(GRAV_E_ARG, "Plummer: need G > 0");
		if (!scratch) return record_error(GRAV_E_ARG, "Plummer: NULL scratch "
			"(grav_scenario_scratch_bytes)");
		if (reinterpret_cast<uintptr_t>(scratch) & 7)
			return record_error(GRAV_E_ARG, "scratch must be 8-byte aligned");
		a.ln_lo = std::log(a.p[1]);
		a.ln_hi = std::log(a.p[2]);
		double* part = static_cast<double*>(scratch);
		plummer_mass_kernel<<<ctas, THREADS, 0, st>>>(R, n, a, part);
		plummer_body_kernel<<<ctas, THREADS, 0, st>>>(R, V, n, a, part);
		plummer_shift_kernel<<<ctas, THREADS, 0, st>>>(R, V, n, a, part);
		break;
	}
	case GRAV_SCEN_GALAXY:
		if (!(a.p[0] > 0.0 && a.p[1] >= 0.0 && a.p[2] >= 0.0 && a.p[3] > 0.0 && a.p[4] > 0.0))
			return record_error(GRAV_E_ARG, "galaxy: need radius > 0, masses >= 0, scales > 0");
		galaxy_kernel<<<ctas, THREADS, 0, st>>>(R, V, n, a);
		break;
	default:
		return record_error(GRAV_E_ARG, "unknown scenario kind");
	}
	const cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return record_error(GRAV_E_CUDA, cudaGetErrorString(e));
	return GRAV_OK;
}

}  // extern "C"
