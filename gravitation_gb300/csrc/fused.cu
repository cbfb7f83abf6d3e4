// fused.cu -- one full step (stage 1 + stage 2) of one small universe in one launch.
//
// Below a few thousand bodies a step costs little arithmetic, and the two dependent
// launches of the regular path (the persistent stage-1 grid, then stage 2 summing its
// partial-sum slots) set its time: ~8-9 us at 16-512 bodies on GB300, nearly all launch,
// drain and memory latency.  Here each CTA copies every body's FP32 position (and low
// part) into shared memory, completes the accelerations of its own R rows over all
// columns (no partial sums leave the CTA), and integrates those rows in FP64 exactly as
// stage2.cu does.  A row's results are only written once every CTA has finished reading
// the positions.  One CTA needs nothing more than its own __syncthreads.  A grid of up to
// 16 CTAs is one thread-block cluster and uses the hardware cluster barrier (arrive right
// after the copy, wait right before the writes, so it normally costs nothing).  A larger
// grid is a cooperative launch, so all its CTAs are resident together, and uses a grid
// barrier on two device counters that the last CTA to leave resets; its wait is bounded
// all the same (GRAV_WAIT_NS), after which the CTA records GRAV_DEV_TIMEOUT, writes
// nothing and returns.
//
// Work inside a CTA: warps take items (32-row group g, column split s) of the rows it
// holds; the columns are cut into as many splits as leave every warp an item, so that a
// few rows still keep all warps busy, each on a short column range.  Each lane holds one
// row; the pair terms are those of stage1_f32.cu (FP32 separations, rsqrt on the SFU, r2
// floored by eps2; GRAV_MODE_FP32C: double-single separations; GRAV_MODE_FP32N: pairs
// closer than the near radius evaluated again from the double-single separation) and
// every 32 columns the FP32 partials are folded into compensated (TwoSum) sums.  The
// splits' (hi, lo) sums go through shared memory and are combined in a fixed pairwise
// tree: the result does not depend on scheduling.
#include "grav_device.cuh"

namespace grav {

enum { FUSED_PLAIN = 0, FUSED_DS = 1, FUSED_NEAR = 2 };
constexpr unsigned FUSED_CLUSTER_PORTABLE = 8;   // portable thread-block cluster size
constexpr unsigned FUSED_CLUSTER_MAX = 16;       // largest, where the GPU schedules it

struct __align__(32) frow4 {
	double x, y, z, w;
};

// 16-byte asynchronous copy global -> shared (bypassing L1), and the wait for all of a
// thread's outstanding copies (the data is then visible to that thread)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(smem)), "l"(gmem)
		: "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
	asm volatile("cp.async.wait_all;" ::: "memory");
}

// CTAs in this CTA's thread-block cluster (1 when launched without clusters)
__device__ __forceinline__ unsigned cluster_ctas()
{
	unsigned v;
	asm("mov.u32 %0, %%cluster_nctarank;" : "=r"(v));
	return v;
}

// Hardware cluster barrier, split: every thread of every CTA of the cluster arrives
// (release: its earlier loads and stores are ordered before) and later waits (acquire).
__device__ __forceinline__ void cluster_arrive()
{
	asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}

__device__ __forceinline__ void cluster_wait()
{
	asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Bytes of dynamic shared memory: positions (and low parts) of n bodies padded to a
// multiple of 4; the splits' compensated sums, 3 components x (hi, lo) for splits x
// row groups <= warps items of 32 rows; the rows' FP64 state (r, v), staged by cp.async.
__host__ __device__ inline int64_t fused_smem_bytes(int np, int64_t n, int threads, int rows)
{
	const int64_t npad = (n + 3) / 4 * 4;
	const int64_t r32 = (rows + 31) / 32 * 32;
	return np * npad * 16 + static_cast<int64_t>(threads / 32) * 3 * 32 * 8 + r32 * 64;
}

// Stage 2 of one row: a_out, the FP64 update and the row of the stage-1 positions.
template <int NP>
__device__ __forceinline__ void write_row(const grav_batch& b, int flags, double Tu,
	int il, int64_t row, double ax, double ay, double az, const frow4* st, frow4* rr, frow4* vv)
{
	frow4 r = st[0];
	if ((flags & GRAV_S2_WRITE_A) && b.a_out) {
		double2* ao = reinterpret_cast<double2*>(b.a_out) + 2 * row;
		__stcs(ao, make_double2(ax, ay));
		__stcs(ao + 1, make_double2(az, 0.0));
	}
	if (flags & GRAV_S2_INTEGRATE) {
		// the base class's update with separately rounded products and sums
		// (_base_.py:58-62, np2.py:110-115), as stage2.cu applies it
		frow4 v = st[1];
		v.x = __dadd_rn(__dmul_rn(ax, Tu), v.x);
		v.y = __dadd_rn(__dmul_rn(ay, Tu), v.y);
		v.z = __dadd_rn(__dmul_rn(az, Tu), v.z);
		r.x = __dadd_rn(__dmul_rn(v.x, Tu), r.x);
		r.y = __dadd_rn(__dmul_rn(v.y, Tu), r.y);
		r.z = __dadd_rn(__dmul_rn(v.z, Tu), r.z);
		vv[row] = v;
		rr[row] = r;
	}
	// the row of the stage-1 position array, as stage2.cu writes it
	float4* q = static_cast<float4*>(b.pos);
	const float qx = __double2float_rn(r.x);
	const float qy = __double2float_rn(r.y);
	const float qz = __double2float_rn(r.z);
	q[il] = make_float4(qx, qy, qz, __double2float_rn(r.w));
	if (NP == 2)
		q[b.n_pad_total + il] = make_float4(__double2float_rn(__dsub_rn(r.x, static_cast<double>(qx))),
			__double2float_rn(__dsub_rn(r.y, static_cast<double>(qy))),
			__double2float_rn(__dsub_rn(r.z, static_cast<double>(qz))), 0.f);
}

template <int T, int KIND>
__global__ void __launch_bounds__(T) fused_step_kernel(const grav_batch b, const int flags,
	const int R, int32_t* __restrict__ sync)
{
	constexpr bool DS = KIND == FUSED_DS;
	constexpr bool NEAR = KIND == FUSED_NEAR;
	constexpr int NP = KIND == FUSED_PLAIN ? 1 : 2;
	constexpr int W = T / 32;
	extern __shared__ __align__(16) float4 fsm[];

	const int tid = threadIdx.x;
	const int lane = tid & 31;
	const int warp = tid >> 5;
	// one universe laid out by grav_plan: its rows start at row 0 of r, v and the
	// position array, so no address waits for the plan table (only T is read from it)
	const double Tu = b.univ[0].T;
	// launched as a programmatic dependent (one CTA or one cluster): the next step may
	// begin launching now, and this one waits here until the kernel before it (the
	// previous step, or the prepare pass) has finished and its writes are visible
	grid_dep_launch();
	grid_dep_wait();
	const int n = static_cast<int>(b.n_bodies);
	const int npad = (n + 3) / 4 * 4;
	const int G = gridDim.x;
	const int row0 = blockIdx.x * R;                       // first local row of this CTA
	const int rows_here = max(0, min(R, n - row0));        // rows this CTA completes
	const int RG = max(1, (rows_here + 31) / 32);          // their 32-row groups
	const int S = W >= RG ? W / RG : 1;                    // column splits (S x RG <= W)
	const int RS = RG * 32;                                // row stride of the split sums
	const int cs = ((npad + S - 1) / S + 3) / 4 * 4;       // columns per split
	const float eps2 = b.eps2;

	float4* __restrict__ sp = fsm;                        // [npad] hi (x, y, z, Gm)
	float4* __restrict__ spl = fsm + (NP == 2 ? npad : 0);  // [npad] lo (DS, NEAR)
	float2* __restrict__ red = reinterpret_cast<float2*>(fsm + NP * npad);  // [S][3][RS]

	// this thread's row of the state (tid < R), copied to shared memory asynchronously
	// now, so that its latency overlaps the position copy and the pair loop (held in
	// registers through the loop it cost spills)
	const int il = row0 + tid;
	const bool mine = tid < rows_here;
	const int64_t row = il;
	frow4* rr = reinterpret_cast<frow4*>(b.r);
	frow4* vv = reinterpret_cast<frow4*>(b.v);
	frow4* st = reinterpret_cast<frow4*>(red + W * 3 * 32) + 2 * tid;
	if (mine) {
		cp_async16(reinterpret_cast<char*>(st), reinterpret_cast<const char*>(rr + row));
		cp_async16(reinterpret_cast<char*>(st) + 16, reinterpret_cast<const char*>(rr + row) + 16);
		if (flags & GRAV_S2_INTEGRATE) {
			cp_async16(reinterpret_cast<char*>(st + 1), reinterpret_cast<const char*>(vv + row));
			cp_async16(reinterpret_cast<char*>(st + 1) + 16,
				reinterpret_cast<const char*>(vv + row) + 16);
		}
	}

	// ---- positions of every body -> shared memory (padding columns: zero, Gm = 0) ----
	const float4* __restrict__ pos = static_cast<const float4*>(b.pos);
	const float4* __restrict__ poslo = static_cast<const float4*>(b.pos) + b.n_pad_total;
	for (int i = tid; i < npad; i += T) {
		const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
		sp[i] = i < n ? pos[i] : z;
		if (NP == 2) spl[i] = i < n ? poslo[i] : z;
	}
	__syncthreads();
	// every read of the positions this CTA makes is done: arrive.  One CTA alone needs no
	// barrier (its own __syncthreads orders its reads before its writes); a grid that is
	// one thread-block cluster uses the cluster's hardware barrier; a larger grid the
	// counters in `sync`
	const bool clustered = G > 1 && cluster_ctas() == static_cast<unsigned>(G);
	const bool counters = G > 1 && !clustered;
	if (clustered) cluster_arrive();
	if (counters && tid == 0) {
		__threadfence();
		atomicAdd(&sync[0], 1);
	}

	// ---- accelerations of this CTA's rows: item (row group g, split s) per warp ----
	for (int item = warp; item < RG * S; item += W) {
		const int g = item % RG, s = item / RG;
		const int li = g * 32 + lane;        // row within the CTA
		const int il = row0 + li;            // row within the universe
		const bool real = li < rows_here;
		const float4 pi = sp[real ? il : 0];
		const float4 qi = NP == 2 ? spl[real ? il : 0] : make_float4(0.f, 0.f, 0.f, 0.f);
		const float thr = NEAR ? near_threshold(near_scale(pi.x, pi.y, pi.z)) : 0.f;
		float hx = 0.f, hy = 0.f, hz = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
		const int c0 = min(npad, s * cs), c1 = min(npad, c0 + cs);
		// the split's columns in blocks of up to 32, each folded into the compensated sums
		for (int cb = c0; cb < c1; cb += 32) {
			float fx = 0.f, fy = 0.f, fz = 0.f;
			const float4* __restrict__ sc = sp + cb;
			const float4* __restrict__ scl = spl + cb;
			const int nj = min(32, c1 - cb);   // a multiple of 4
			// with the near test's vote in every step the loop is not unrolled (unrolled by
			// 4 it measured 2-3 % slower at 16-256 bodies)
#pragma unroll (NEAR ? 1 : 4)
			for (int j = 0; j < nj; ++j) {
				const float4 pj = sc[j];
				float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
				if (DS) {
					const float4 lj = scl[j];
					dx = dx + (lj.x - qi.x);
					dy = dy + (lj.y - qi.y);
					dz = dz + (lj.z - qi.z);
				}
				const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
				const float inv = rsqrt_sfu(r2);
				float w = pj.w * inv;
				w = w * (inv * inv);
				fx = fmaf(dx, w, fx);
				fy = fmaf(dy, w, fy);
				fz = fmaf(dz, w, fz);
				if (NEAR) {
					// the self pair and coincident bodies (r2 = eps2) are not near pairs
					const bool nk = (r2 < thr) & (r2 > eps2);
					if (__any_sync(0xffffffffu, nk)) {
						float ex, ey, ez;
						near_delta(dx, dy, dz, r2, scl[j], qi, eps2, nk, ex, ey, ez);
						fx = fmaf(ex, pj.w, fx);
						fy = fmaf(ey, pj.w, fy);
						fz = fmaf(ez, pj.w, fz);
					}
				}
			}
			two_sum_acc(hx, lx, fx);
			two_sum_acc(hy, ly, fy);
			two_sum_acc(hz, lz, fz);
		}
		float2* rs = red + s * 3 * RS + li;
		rs[0] = make_float2(hx, lx);
		rs[RS] = make_float2(hy, ly);
		rs[2 * RS] = make_float2(hz, lz);
	}
	__syncthreads();

	// ---- the splits' compensated sums, combined pairwise in a fixed tree: split s takes
	// split s + h (h = half the live splits, rounded up) until one is left ----
	for (int live = S; live > 1;) {
		const int h = (live + 1) / 2;
		const int m = (live - h) * 3 * RS;  // entries combined in this round
		for (int e = tid; e < m; e += T) {
			float2* a = red + e;
			const float2 b2 = a[h * 3 * RS];
			float2 a2 = *a;
			two_sum_acc(a2.x, a2.y, b2.x);
			a2.y += b2.y;
			*a = a2;
		}
		live = h;
		__syncthreads();
	}
	// ---- one thread per row: widened once ----
	double ax = 0.0, ay = 0.0, az = 0.0;
	if (mine) {
		const float2 px = red[tid], py = red[RS + tid], pz = red[2 * RS + tid];
		ax = static_cast<double>(px.x) + static_cast<double>(px.y);
		ay = static_cast<double>(py.x) + static_cast<double>(py.y);
		az = static_cast<double>(pz.x) + static_cast<double>(pz.y);
	}

	// ---- wait until every CTA has read the positions, then write ----
	__shared__ int timed_out;
	if (tid == 0) {
		bool ok = true;
		if (counters) {
			volatile int32_t* arrived = sync;
			ok = *arrived >= G;
			if (!ok) {
				const uint64_t t0 = global_ns();
				for (;;) {
					for (int k = 0; k < 16 && !ok; ++k) ok = *arrived >= G;
					if (ok || global_ns() - t0 > GRAV_WAIT_NS) break;
				}
			}
			__threadfence();
			if (!ok) set_error(b.err, GRAV_DEV_TIMEOUT);
		}
		timed_out = ok ? 0 : 1;
	}
	__syncthreads();
	if (clustered) cluster_wait();
	cp_async_wait_all();
	if (!timed_out && mine) write_row<NP>(b, flags, Tu, il, row, ax, ay, az, st, rr, vv);
	// leave; the last CTA out resets both counters for the next launch
	if (counters && tid == 0 && atomicAdd(&sync[1], 1) == G - 1) {
		sync[0] = 0;
		sync[1] = 0;
		__threadfence();
	}
}

struct FusedKernel {
	int mode, threads;
	const void* fn;
};

#define GRAV_FUSED_ENTRY(M, T, K) {M, T, reinterpret_cast<const void*>(&fused_step_kernel<T, K>)}

static const FusedKernel k_fused[] = {
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32, 256, FUSED_PLAIN),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32, 512, FUSED_PLAIN),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32, 1024, FUSED_PLAIN),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32C, 256, FUSED_DS),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32C, 512, FUSED_DS),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32C, 1024, FUSED_DS),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32N, 256, FUSED_NEAR),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32N, 512, FUSED_NEAR),
	GRAV_FUSED_ENTRY(GRAV_MODE_FP32N, 1024, FUSED_NEAR),
};

const void* find_fused(int mode, int threads)
{
	for (const FusedKernel& k : k_fused)
		if (k.mode == mode && k.threads == threads) return k.fn;
	return nullptr;
}

int64_t fused_smem(int mode, int64_t n, int threads, int rows)
{
	return fused_smem_bytes(mode == GRAV_MODE_FP32 ? 1 : 2, n, threads, rows);
}

// A grid of one CTA has no barrier and launches the ordinary way.  Up to 16 CTAs launch
// as one thread-block cluster (co-scheduled by the hardware; the kernel then uses the
// cluster barrier; above 8 CTAs only where the occupancy query finds room for such a
// cluster), more as a cooperative launch (all CTAs resident at once, or the launch
// fails), which the kernel's counter barrier relies on.  On GB300 a cooperative launch
// measured ~0.5 us more per graph node, and the counter barrier ~1 us more than the
// cluster barrier.  One CTA and one cluster also launch as programmatic dependents, so
// that a step's launch overlaps the end of the one before (0.3-0.6 us per step at 16-512
// bodies); the cooperative grid does not (its CTAs must all be resident at once).
cudaError_t launch_fused(const grav_batch& b, int flags, int threads, int rows, int32_t* sync,
	cudaStream_t stream)
{
	const void* fn = find_fused(b.mode, threads);
	const int64_t smem = fused_smem(b.mode, b.n_bodies, threads, rows);
	cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
		static_cast<int>(smem));
	if (e != cudaSuccess) return e;
	const unsigned grid = static_cast<unsigned>((b.n_bodies + rows - 1) / rows);
	grav_batch copy = b;
	int f = flags, R = rows;
	int32_t* s = sync;
	void* args[] = {&copy, &f, &R, &s};
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(threads);
	cfg.dynamicSmemBytes = static_cast<size_t>(smem);
	cfg.stream = stream;
	cudaLaunchAttribute attr[2];
	cfg.attrs = attr;
	cfg.numAttrs = grid > 1 ? 1 : 0;
	bool cluster = grid > 1 && grid <= FUSED_CLUSTER_MAX;
	if (cluster) {
		attr[0].id = cudaLaunchAttributeClusterDimension;
		attr[0].val.clusterDim.x = grid;
		attr[0].val.clusterDim.y = 1;
		attr[0].val.clusterDim.z = 1;
		if (grid > FUSED_CLUSTER_PORTABLE) {
			int fits = 0;
			e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
			if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&fits, fn, &cfg);
			if (e != cudaSuccess) {
				cudaGetLastError();  // a refused query is not sticky: fall back
				fits = 0;
			}
			cluster = fits > 0;
		}
	}
	if (grid > 1 && !cluster) {
		attr[0].id = cudaLaunchAttributeCooperative;
		attr[0].val.cooperative = 1;
	} else {
		attr[cfg.numAttrs].id = cudaLaunchAttributeProgrammaticStreamSerialization;
		attr[cfg.numAttrs].val.programmaticStreamSerializationAllowed = 1;
		++cfg.numAttrs;
	}
	return cudaLaunchKernelExC(&cfg, fn, args);
}

int fused_occupancy(int mode, int64_t n, int threads, int rows, int* ctas_per_sm)
{
	const void* fn = find_fused(mode, threads);
	if (!fn) return -1;
	const int64_t smem = fused_smem(mode, n, threads, rows);
	cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
		static_cast<int>(smem));
	if (e != cudaSuccess) return -2;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, threads,
		static_cast<size_t>(smem));
	return e == cudaSuccess ? 0 : -2;
}

}  // namespace grav
