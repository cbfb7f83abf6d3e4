/*
 * scenario.c -- CPU restatement of the seeded scenario generator (TEST INFRASTRUCTURE
 * ONLY: tests/ use it as the checker of the device generator; the product never links
 * it).  Compiled into liboracle.so with -ffp-contract=off, so every product and sum
 * below is one rounded IEEE operation, as the device code writes them.
 *
 * Generator: Philox4x64-10 (Salmon, Moraes, Dror, Shaw, SC'11), key {seed, stream},
 * counter {body, block, 0, 0}; uniform double = (word >> 11) * 2^-53.  Pinned in the
 * tests against numpy's own Philox bit generator (numpy.random.Philox, the same
 * 4x64-10 algorithm; numpy advances its counter before it draws a block).
 *
 * Scenarios:
 *   1 uniform cube  r ~ U[-h, h]^3, v ~ N(0, sigma^2)^3 by Box-Muller, m ~ U[lo, hi]
 *   2 Plummer       Aarseth, Henon & Wielen (1974, A&A 37, 183): radius from the
 *                   inverted cumulative mass cut at 99.9 %, speed q v_esc(r) with q from
 *                   q^2 (1 - q^2)^(7/2) by rejection, masses log-uniform; then the centre
 *                   of mass is moved to (cx, cy, cz) with velocity (cvx, cvy, cvz).  The
 *                   sums run in body order here (a fixed tree on the device), so those
 *                   bodies agree to rounding, not bit for bit.
 *   3 galaxy        gravitation/lib/simulation.py:99-184 (create_galaxy: disc of the
 *                   first 4/5 of the stars, bulge of the rest, circular speeds about the
 *                   central mass with the universe's scaled G, simulation.py:147-149),
 *                   with the zero rotations left out, scaled as add_object scales
 *                   (gravitation/kernel/_base_.py:114-117).
 */
#include <math.h>
#include <stdint.h>

#define PHILOX_M0 0xD2E7470EE14C6C93ull
#define PHILOX_M1 0xCA5A826395121157ull
#define PHILOX_W0 0x9E3779B97F4A7C15ull
#define PHILOX_W1 0xBB67AE8584CAA73Bull

static const double TWO_PI = 6.283185307179586;
static const double PI_ = 3.141592653589793;
static const double HALF_PI = 1.5707963267948966;
static const double Q_FALLBACK = 0.4714045207910317;

void orc_philox4x64_10(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4])
{
	uint64_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3], k0 = key[0], k1 = key[1];
	for (int round = 0; round < 10; round++) {
		const unsigned __int128 p0 = (unsigned __int128)PHILOX_M0 * x0;
		const unsigned __int128 p1 = (unsigned __int128)PHILOX_M1 * x2;
		const uint64_t hi0 = (uint64_t)(p0 >> 64), lo0 = (uint64_t)p0;
		const uint64_t hi1 = (uint64_t)(p1 >> 64), lo1 = (uint64_t)p1;
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

static void draw(int64_t i, uint64_t block, uint64_t seed, uint64_t stream, uint64_t w[4])
{
	const uint64_t c[4] = {(uint64_t)i, block, 0, 0}, k[2] = {seed, stream};
	orc_philox4x64_10(c, k, w);
}

static inline double u01(uint64_t w) { return (double)(w >> 11) * 0x1.0p-53; }

static inline double lin(double lo, double hi, double u) { return lo + (hi - lo) * u; }

static void isotropic(double uc, double up, double rad, double *x, double *y, double *z)
{
	*z = (1.0 - 2.0 * uc) * rad;
	const double phi = TWO_PI * up;
	const double rho = sqrt(fmax(rad * rad - *z * *z, 0.0));
	*x = rho * cos(phi);
	*y = rho * sin(phi);
}

static void cube(uint64_t seed, uint64_t stream, double G, const double *p, int64_t n,
	double *r, double *v)
{
	const double h = p[0], sigma = p[1];
	for (int64_t i = 0; i < n; i++) {
		uint64_t w[4], u[4];
		draw(i, 0, seed, stream, w);
		draw(i, 1, seed, stream, u);
		double *R = r + 4 * i, *V = v + 4 * i;
		R[0] = lin(-h, h, u01(w[0]));
		R[1] = lin(-h, h, u01(w[1]));
		R[2] = lin(-h, h, u01(w[2]));
		R[3] = G * lin(p[2], p[3], u01(w[3]));
		const double rad0 = sqrt(-2.0 * log(1.0 - u01(u[0])));
		const double th0 = TWO_PI * u01(u[1]);
		const double rad1 = sqrt(-2.0 * log(1.0 - u01(u[2])));
		const double th1 = TWO_PI * u01(u[3]);
		V[0] = sigma * (rad0 * cos(th0));
		V[1] = sigma * (rad0 * sin(th0));
		V[2] = sigma * (rad1 * cos(th1));
		V[3] = 0.0;
	}
}

static void plummer(uint64_t seed, uint64_t stream, double G, const double *p, int64_t n,
	double *r, double *v)
{
	const double a = p[0], ln_lo = log(p[1]), ln_hi = log(p[2]);
	double gm_tot = 0.0;
	for (int64_t i = 0; i < n; i++) {
		uint64_t w[4];
		draw(i, 0, seed, stream, w);
		r[4 * i + 3] = G * exp(lin(ln_lo, ln_hi, u01(w[0])));
		gm_tot += r[4 * i + 3];
	}
	const double vesc0 = sqrt(2.0 * gm_tot / a);
	double s[6] = {0, 0, 0, 0, 0, 0};
	for (int64_t i = 0; i < n; i++) {
		uint64_t w[4], d[4];
		draw(i, 0, seed, stream, w);
		draw(i, 1, seed, stream, d);
		double *R = r + 4 * i, *V = v + 4 * i;
		const double X = lin(1e-10, 0.999, u01(w[1]));
		const double rad = a / sqrt(expm1((-2.0 / 3.0) * log(X)));
		isotropic(u01(w[2]), u01(w[3]), rad, &R[0], &R[1], &R[2]);
		double q = Q_FALLBACK;
		int found = 0;
		for (int blk = 2; blk < 2 + 32 && !found; blk++) {
			uint64_t t[4];
			draw(i, (uint64_t)blk, seed, stream, t);
			for (int k = 0; k < 4 && !found; k += 2) {
				const double x4 = u01(t[k]), x5 = u01(t[k + 1]);
				const double x2 = x4 * x4, y = 1.0 - x2;
				const double g = (x2 * ((y * y) * y)) * sqrt(y);
				if (0.1 * x5 < g) {
					q = x4;
					found = 1;
				}
			}
		}
		const double xr = rad / a;
		const double ve = vesc0 / sqrt(sqrt(1.0 + xr * xr));
		isotropic(u01(d[0]), u01(d[1]), q * ve, &V[0], &V[1], &V[2]);
		V[3] = 0.0;
		for (int k = 0; k < 3; k++) {
			s[k] += R[3] * R[k];
			s[3 + k] += R[3] * V[k];
		}
	}
	for (int k = 0; k < 6; k++) s[k] = s[k] / gm_tot;
	for (int64_t i = 0; i < n; i++)
		for (int k = 0; k < 3; k++) {
			r[4 * i + k] = (r[4 * i + k] - s[k]) + p[3 + k];
			v[4 * i + k] = (v[4 * i + k] - s[3 + k]) + p[6 + k];
		}
}

static void galaxy(uint64_t seed, uint64_t stream, double G, const double *p, int64_t n,
	double *r, double *v)
{
	const double radius = p[0], m_hole = p[1], m_star = p[2], sr = p[3], sm = p[4];
	const int64_t stars = n - 1, n_disc = stars * 4 / 5;
	const double span = (4.5 + 0.1) * radius;
	const double gm_hole = G * m_hole;
	if (n < 1) return;
	r[0] = r[1] = r[2] = 0.0;
	r[3] = G * (m_hole * sm);
	v[0] = v[1] = v[2] = v[3] = 0.0;
	for (int64_t i = 1; i < n; i++) {
		uint64_t w[4];
		draw(i, 0, seed, stream, w);
		const double alpha = (u01(w[0]) * 2.0) * PI_;
		double x, y, z;
		if (i - 1 < n_disc) {
			const double r_abs = (u01(w[1]) * 4.5 + 0.1) * radius;
			x = r_abs * cos(alpha);
			y = r_abs * sin(alpha);
			z = (((0.5 * u01(w[2]) - 0.25) * radius) * (span - r_abs)) / span;
		} else {
			const double r_abs = (u01(w[1]) * 0.75 + 0.1) * radius;
			const double beta = PI_ * (u01(w[2]) - 0.5);
			x = (r_abs * cos(alpha)) * cos(beta);
			y = (r_abs * sin(alpha)) * cos(beta);
			z = r_abs * sin(beta);
		}
		const double dist = sqrt((x * x + y * y) + z * z);
		const double v_abs = sqrt(gm_hole / dist);
		const double va = alpha - HALF_PI;
		double *R = r + 4 * i, *V = v + 4 * i;
		R[0] = x * sr;
		R[1] = y * sr;
		R[2] = z * sr;
		R[3] = G * (m_star * sm);
		V[0] = (v_abs * cos(va)) * sr;
		V[1] = (v_abs * sin(va)) * sr;
		V[2] = V[3] = 0.0;
	}
}

/* r, v: n x 4 doubles.  Returns 0, or -1 for an unknown kind. */
int orc_scenario(int kind, uint64_t seed, uint64_t stream, double G, const double *p,
	int64_t n, double *r, double *v)
{
	switch (kind) {
	case 1: cube(seed, stream, G, p, n, r, v); return 0;
	case 2: plummer(seed, stream, G, p, n, r, v); return 0;
	case 3: galaxy(seed, stream, G, p, n, r, v); return 0;
	default: return -1;
	}
}
