/*
 * oracle.c -- CPU oracle for the all-pairs n-body step (TEST INFRASTRUCTURE ONLY).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm
 * may load this library, and only as the checker or the timed CPU baseline.  The
 * product path (gravitation_gb300) never links or calls it.
 *
 * Restates, in FP64 with compensated (Neumaier) summation, the force law of the
 * reference's own kernels:
 *   gravitation/kernel/np1.py:81-95   (update_pair: rel = r_i - r_j; s = sum rel^2;
 *                                      inv = 1/sqrt(s); rel *= inv; f = G/s;
 *                                      a_i -= rel*f*m_j; a_j += rel*f*m_i)
 *   gravitation/kernel/py1.py:57-64   (same law, pure Python, FP64)
 * the base-class scaling and stage 2:
 *   gravitation/kernel/_base_.py:58-62 (move: v = a*T + v; r = v*T + r; a = 0)
 * and the energy diagnostic that the reference only lists as a wish (TODO.md:4).
 *
 * Compile with -ffp-contract=off so that a*T + v is two rounded operations, exactly
 * as in the reference's Python floats.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Neumaier compensated accumulator */
typedef struct { double s, c; } nsum_t;

static inline void nsum_add(nsum_t *a, double x)
{
	double t = a->s + x;
	if (fabs(a->s) >= fabs(x))
		a->c += (a->s - t) + x;
	else
		a->c += (x - t) + a->s;
	a->s = t;
}

static inline double nsum_get(const nsum_t *a) { return a->s + a->c; }

int orc_abi_version(void) { return 1; }

/*
 * Accelerations of the listed rows in FP64.
 *   r: n x 3 positions (row major), m: n masses, G: already-scaled constant
 *   rows: nrows body indices (NULL = all bodies, nrows must then equal n)
 *   a_out: nrows x 3
 *   coincident: 0 -> follow the reference (a distinct body at zero distance gives
 *               inf/nan, np1.py:85-88 divides by zero); 1 -> skip such pairs.
 * The self pair (j == i) is always excluded, as in np1/py1 which only visit j != i.
 */
void orc_accel_fp64(const double *r, const double *m, double G, int64_t n,
	const int64_t *rows, int64_t nrows, double *a_out, int coincident, int threads)
{
	if (threads < 1) threads = 1;
	#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
	for (int64_t k = 0; k < nrows; k++) {
		const int64_t i = rows ? rows[k] : k;
		nsum_t ax = {0, 0}, ay = {0, 0}, az = {0, 0};
		const double xi = r[3 * i], yi = r[3 * i + 1], zi = r[3 * i + 2];
		for (int64_t j = 0; j < n; j++) {
			if (j == i) continue;
			const double rx = xi - r[3 * j], ry = yi - r[3 * j + 1], rz = zi - r[3 * j + 2];
			const double s = rx * rx + ry * ry + rz * rz;
			if (coincident && s == 0.0) continue;
			const double inv = 1.0 / sqrt(s);
			const double f = G / s;
			const double a1 = f * m[j];
			nsum_add(&ax, -(rx * inv) * a1);
			nsum_add(&ay, -(ry * inv) * a1);
			nsum_add(&az, -(rz * inv) * a1);
		}
		a_out[3 * k] = nsum_get(&ax);
		a_out[3 * k + 1] = nsum_get(&ay);
		a_out[3 * k + 2] = nsum_get(&az);
	}
}

/* Stage 2 of the base class (_base_.py:58-62), FP64, in place. */
void orc_stage2_fp64(double *r, double *v, const double *a, double T, int64_t n3)
{
	for (int64_t k = 0; k < n3; k++) {
		const double at = a[k] * T;
		v[k] = at + v[k];
		const double vt = v[k] * T;
		r[k] = vt + r[k];
	}
}

/*
 * Energy and momentum in FP64:
 *   out[0] = kinetic   sum 1/2 m v^2
 *   out[1] = potential -sum_{i<j} G m_i m_j / |r_i - r_j|
 *   out[2..4] = momentum sum m v
 */
void orc_energy_fp64(const double *r, const double *v, const double *m, double G,
	int64_t n, double *out, int threads)
{
	if (threads < 1) threads = 1;
	double *pot = (double *)calloc((size_t)n, sizeof(double));
	#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
	for (int64_t i = 0; i < n; i++) {
		nsum_t p = {0, 0};
		for (int64_t j = i + 1; j < n; j++) {
			const double dx = r[3 * i] - r[3 * j], dy = r[3 * i + 1] - r[3 * j + 1],
				dz = r[3 * i + 2] - r[3 * j + 2];
			const double d = sqrt(dx * dx + dy * dy + dz * dz);
			nsum_add(&p, -G * m[i] * m[j] / d);
		}
		pot[i] = nsum_get(&p);
	}
	nsum_t k = {0, 0}, p = {0, 0}, px = {0, 0}, py = {0, 0}, pz = {0, 0};
	for (int64_t i = 0; i < n; i++) {
		const double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
		nsum_add(&k, 0.5 * m[i] * (vx * vx + vy * vy + vz * vz));
		nsum_add(&p, pot[i]);
		nsum_add(&px, m[i] * vx);
		nsum_add(&py, m[i] * vy);
		nsum_add(&pz, m[i] * vz);
	}
	free(pot);
	out[0] = nsum_get(&k);
	out[1] = nsum_get(&p);
	out[2] = nsum_get(&px);
	out[3] = nsum_get(&py);
	out[4] = nsum_get(&pz);
}

/*
 * Discrete adjoint of one symplectic-Euler step (FP64, all pairs), used to check the
 * GPU adjoint kernels on small cases.  With A_i(r) = sum_j G m_j f(r_j - r_i),
 * f(d) = d/|d|^3 and Jf(d) = I/|d|^3 - 3 d d^T/|d|^5:
 *   h_k   = sum_{j!=k} Jf(r_j - r_k) (G m_k u_j - G m_j u_k)     (= J_A(r)^T u)
 *   gmk_k = sum_{j!=k} u_j . (r_j - r_k) / |r_j - r_k|^3          (dA/dm folded)
 * Outputs are n x 3 (h) and n (gmk).
 */
void orc_vjp_fp64(const double *r, const double *m, double G, const double *u,
	int64_t n, double *h, double *gmk, int threads)
{
	if (threads < 1) threads = 1;
	#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
	for (int64_t k = 0; k < n; k++) {
		nsum_t hx = {0, 0}, hy = {0, 0}, hz = {0, 0}, g = {0, 0};
		for (int64_t j = 0; j < n; j++) {
			if (j == k) continue;
			const double dx = r[3 * j] - r[3 * k], dy = r[3 * j + 1] - r[3 * k + 1],
				dz = r[3 * j + 2] - r[3 * k + 2];
			const double s = dx * dx + dy * dy + dz * dz;
			const double inv = 1.0 / sqrt(s);
			const double inv3 = inv / s, inv5 = inv3 / s;
			const double wx = G * m[k] * u[3 * j] - G * m[j] * u[3 * k];
			const double wy = G * m[k] * u[3 * j + 1] - G * m[j] * u[3 * k + 1];
			const double wz = G * m[k] * u[3 * j + 2] - G * m[j] * u[3 * k + 2];
			const double dw = dx * wx + dy * wy + dz * wz;
			nsum_add(&hx, wx * inv3 - 3.0 * dw * inv5 * dx);
			nsum_add(&hy, wy * inv3 - 3.0 * dw * inv5 * dy);
			nsum_add(&hz, wz * inv3 - 3.0 * dw * inv5 * dz);
			nsum_add(&g, (u[3 * j] * dx + u[3 * j + 1] * dy + u[3 * j + 2] * dz) * inv3);
		}
		h[3 * k] = nsum_get(&hx);
		h[3 * k + 1] = nsum_get(&hy);
		h[3 * k + 2] = nsum_get(&hz);
		gmk[k] = nsum_get(&g);
	}
}
