/*
 * ref_port.c -- portable restatement of the reference's fastest CPU stage 1
 * (TEST / BASELINE INFRASTRUCTURE ONLY: timed as the CPU baseline, never shipped).
 *
 * The reference's fastest CPU kernel is c4a (gravitation/kernel/_lib4_/lib.c:76-380):
 * FP32, unique pairs i<j with the symmetric update, OpenMP threads over row segments
 * balanced by pair count (lib.c:76-144), per-thread private accumulators
 * (lib.c:179-182, 289-291), and a serial reduction over threads (lib.c:340-374).
 * Its inner loop is x86 SSE (lib.c:39, 192-317) and does not build on an Arm host,
 * so this file restates the same design in plain C that the compiler vectorises for
 * whatever SIMD the host has.  The per-pair arithmetic follows the portable C kernel
 * (gravitation/kernel/_lib1_/lib.c:78-114) and cy4 (cy4/core.pyx:61-88):
 *   d = r_i - r_j; s = |d|^2; f = G/s; inv = 1/sqrt(s); dn = d*inv;
 *   a_j += dn*f*m_i; a_i -= dn*f*m_j.
 * The row partition follows the idea of cy4/wrapper.py:71-90 (equal pair counts).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int port_abi_version(void) { return 1; }

/* Row boundaries bounds[0..threads] splitting rows [row0, row1) so that each segment
 * holds about the same number of unique pairs (row i owns n-1-i pairs). */
void port_segments(int64_t n, int64_t row0, int64_t row1, int threads, int64_t *bounds)
{
	double total = 0.0;
	for (int64_t i = row0; i < row1; i++) total += (double)(n - 1 - i);
	int64_t row = row0;
	double acc = 0.0;
	bounds[0] = row0;
	for (int t = 1; t < threads; t++) {
		const double goal = total * (double)t / (double)threads;
		while (row < row1 && acc + (double)(n - 1 - row) <= goal) {
			acc += (double)(n - 1 - row);
			row++;
		}
		bounds[t] = row;
	}
	bounds[threads] = row1;
}

/*
 * Stage 1 over the rows [row0, row1) of the pair triangle (all rows: 0, n).
 * x,y,z,m: n floats; ax,ay,az: n floats (overwritten with the result);
 * work: threads * 3 * n floats of scratch (private accumulators).
 */
void port_stage1_rows(const float *x, const float *y, const float *z, const float *m,
	float G, int64_t n, int64_t row0, int64_t row1, float *ax, float *ay, float *az,
	float *work, int threads)
{
	if (threads < 1) threads = 1;
	int64_t *bounds = (int64_t *)malloc(sizeof(int64_t) * (size_t)(threads + 1));
	port_segments(n, row0, row1, threads, bounds);
	memset(work, 0, sizeof(float) * 3 * (size_t)n * (size_t)threads);
	#pragma omp parallel num_threads(threads)
	{
		int t = 0;
#ifdef _OPENMP
		t = omp_get_thread_num();
#endif
		float *px = work + (size_t)t * 3 * (size_t)n;
		float *py = px + n;
		float *pz = py + n;
		for (int64_t i = bounds[t]; i < bounds[t + 1]; i++) {
			const float xi = x[i], yi = y[i], zi = z[i], mi = m[i];
			float sx = 0.f, sy = 0.f, sz = 0.f;
			for (int64_t j = i + 1; j < n; j++) {
				const float dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
				const float s = dx * dx + dy * dy + dz * dz;
				const float f = G / s;
				const float inv = 1.0f / sqrtf(s);
				const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
				const float aj = f * mi, ai = f * m[j];
				px[j] += nx * aj;
				py[j] += ny * aj;
				pz[j] += nz * aj;
				sx -= nx * ai;
				sy -= ny * ai;
				sz -= nz * ai;
			}
			px[i] += sx;
			py[i] += sy;
			pz[i] += sz;
		}
	}
	/* serial reduction over threads, as lib.c:340-374 */
	for (int64_t i = 0; i < n; i++) {
		float sx = 0.f, sy = 0.f, sz = 0.f;
		for (int t = 0; t < threads; t++) {
			const float *px = work + (size_t)t * 3 * (size_t)n;
			sx += px[i];
			sy += px[n + i];
			sz += px[2 * n + i];
		}
		ax[i] = sx;
		ay[i] = sy;
		az[i] = sz;
	}
	free(bounds);
}

/* Base-class stage 2 in FP32 arrays (the reference's c4a inherits the Python stage 2,
 * _base_.py:152-156; here on float arrays like np2.py:110-115). */
void port_stage2(float *x, float *y, float *z, float *vx, float *vy, float *vz,
	const float *ax, const float *ay, const float *az, float T, int64_t n)
{
	for (int64_t i = 0; i < n; i++) {
		vx[i] += ax[i] * T;
		vy[i] += ay[i] * T;
		vz[i] += az[i] * T;
		x[i] += vx[i] * T;
		y[i] += vy[i] * T;
		z[i] += vz[i] * T;
	}
}
