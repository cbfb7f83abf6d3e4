// abi.cu -- the extern "C" entry points of libgravgb300.so.
//
// Validation happens on the host before anything is queued on the GPU, so argument
// errors never reach a kernel.  The library keeps no global mutable state apart from
// the thread-local message of the last failure.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "grav_types.h"

namespace {

thread_local std::string g_last_error = "no error";

int fail(int code, const char* fmt, ...)
{
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_last_error = buf;
	return code;
}

int ok()
{
	return GRAV_OK;
}

int cuda_fail(cudaError_t e, const char* what)
{
	return fail(GRAV_E_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

int stage1_table_for(int mode, const grav::Stage1Kernel** tab)
{
	if (mode == GRAV_MODE_FP64) return grav::stage1_table_f64(tab);
	if (mode == GRAV_MODE_FP32U || mode == GRAV_MODE_FP32CU || mode == GRAV_MODE_FP32UN)
		return grav::stage1_table_sym(tab);
	return grav::stage1_table_f32(tab);
}

const grav::Stage1Kernel* find_kernel(int mode, int bpt, int threads, int jtile)
{
	const grav::Stage1Kernel* tab = nullptr;
	int n = stage1_table_for(mode, &tab);
	for (int i = 0; i < n; ++i)
		if (tab[i].mode == mode && tab[i].bpt == bpt && tab[i].threads == threads &&
			tab[i].jtile == jtile)
			return &tab[i];
	return nullptr;
}

// Raise a kernel's dynamic shared-memory limit to what its launch asks for, once per
// kernel and device: static plus dynamic shared memory above 48 KB (the near-pair
// kernels' row buffers) needs the opt-in.  Called before occupancy queries and launches.
cudaError_t ensure_smem(const grav::Stage1Kernel* k)
{
	static std::mutex mu;
	static std::set<std::pair<int, const void*>> done;
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	std::lock_guard<std::mutex> lock(mu);
	if (done.count({dev, k->fn})) return cudaSuccess;
	e = cudaFuncSetAttribute(k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, k->smem_bytes);
	if (e == cudaSuccess) done.insert({dev, k->fn});
	return e;
}

bool valid_mode(int mode)
{
	return mode == GRAV_MODE_FP32 || mode == GRAV_MODE_FP32C || mode == GRAV_MODE_FP64 ||
		mode == GRAV_MODE_FP32U || mode == GRAV_MODE_FP32CU || mode == GRAV_MODE_FP32N ||
		mode == GRAV_MODE_FP32UN;
}

int check_batch(const grav_batch* b)
{
	if (!b) return fail(GRAV_E_ARG, "grav_batch is NULL");
	if (!valid_mode(b->mode)) return fail(GRAV_E_ARG, "unknown precision mode %d", b->mode);
	if (b->n_univ < 0 || b->n_seg < 0 || b->n_slots < 0 || b->n_bodies < 0 ||
		b->n_pad_total < 0 || b->n_units < 0)
		return fail(GRAV_E_ARG, "negative size in grav_batch");
	const int64_t itile = static_cast<int64_t>(b->tile.bpt) * b->tile.threads;
	if (b->tile.bpt <= 0 || b->tile.threads <= 0 || b->tile.jtile <= 0)
		return fail(GRAV_E_ARG, "tile sizes must be positive");
	if (b->n_pad_total != static_cast<int64_t>(b->n_seg) * itile)
		return fail(GRAV_E_ARG, "n_pad_total (%lld) != n_seg (%d) * itile (%lld)",
			(long long)b->n_pad_total, b->n_seg, (long long)itile);
	if (b->n_pad_total > 0 && (!b->univ || !b->seg || !b->pos || !b->r))
		return fail(GRAV_E_ARG, "NULL device pointer in grav_batch (univ/seg/pos/r)");
	if (b->n_pad_total > 0 && b->n_univ <= 0)
		return fail(GRAV_E_ARG, "rows without universes");
	if (!(b->eps2 > 0.f) && b->mode != GRAV_MODE_FP64)
		return fail(GRAV_E_ARG, "eps2 must be > 0 in the FP32 modes (see grav_eps2)");
	return ok();
}

}  // namespace

namespace grav {
// Message for grav_last_error() from other translation units (failure paths only).
int record_error(int code, const char* msg)
{
	return fail(code, "%s", msg);
}
}  // namespace grav

extern "C" {

int grav_abi_version(void)
{
	return GRAV_ABI_VERSION;
}

const char* grav_last_error(void)
{
	return g_last_error.c_str();
}

int grav_device_query(int device, int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor)
{
	cudaDeviceProp prop;
	cudaError_t e = cudaGetDeviceProperties(&prop, device);
	if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
	if (sm_count) *sm_count = prop.multiProcessorCount;
	if (cc_major) *cc_major = prop.major;
	if (cc_minor) *cc_minor = prop.minor;
	if (!(prop.major == 10 && prop.minor == 3))
		return fail(GRAV_E_DEVICE, "device %d (%s) is compute capability %d.%d; this library "
			"holds sm_103a code only", device, prop.name, prop.major, prop.minor);
	return ok();
}

int grav_tile_supported(int mode, const grav_tile* tile)
{
	if (!tile || !valid_mode(mode)) return 0;
	return find_kernel(mode, tile->bpt, tile->threads, tile->jtile) ? 1 : 0;
}

int grav_tile_list(int mode, grav_tile* out, int cap)
{
	if (!valid_mode(mode)) return fail(GRAV_E_ARG, "unknown precision mode %d", mode);
	const grav::Stage1Kernel* tab = nullptr;
	int n = stage1_table_for(mode, &tab);
	int count = 0;
	for (int i = 0; i < n; ++i) {
		if (tab[i].mode != mode) continue;
		if (out && count < cap) out[count] = grav_tile{tab[i].bpt, tab[i].threads, tab[i].jtile, 0};
		++count;
	}
	return count;
}

int grav_occupancy(int mode, const grav_tile* tile, int32_t* ctas_per_sm)
{
	if (!tile || !ctas_per_sm) return fail(GRAV_E_ARG, "NULL argument");
	if (!valid_mode(mode)) return fail(GRAV_E_ARG, "unknown precision mode %d", mode);
	const grav::Stage1Kernel* k = find_kernel(mode, tile->bpt, tile->threads, tile->jtile);
	if (!k)
		return fail(GRAV_E_TILE, "tile bpt=%d threads=%d jtile=%d not compiled for mode %d",
			tile->bpt, tile->threads, tile->jtile, mode);
	cudaError_t e = ensure_smem(k);
	if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute (dynamic shared memory)");
	int blocks = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k->fn, k->threads, k->smem_bytes);
	if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
	*ctas_per_sm = blocks;
	return ok();
}

int grav_plan(int32_t n_univ, const int32_t* n, const double* T, const grav_tile* tile,
	grav_plan_info* info, grav_univ_desc* univ_out, grav_seg_desc* seg_out)
{
	if (n_univ < 0) return fail(GRAV_E_ARG, "n_univ < 0");
	if (n_univ > 0 && !n) return fail(GRAV_E_ARG, "n is NULL");
	if (!tile || !info) return fail(GRAV_E_ARG, "tile or info is NULL");
	if (tile->bpt <= 0 || tile->threads <= 0 || tile->jtile <= 0 || tile->grid <= 0)
		return fail(GRAV_E_ARG, "tile sizes must be positive");
	const auto pow2 = [](int x) { return x > 0 && (x & (x - 1)) == 0; };
	if (!pow2(tile->bpt) || !pow2(tile->threads) || !pow2(tile->jtile))
		return fail(GRAV_E_ARG, "tile sizes must be powers of two");
	const int64_t itile = static_cast<int64_t>(tile->bpt) * tile->threads;
	const int64_t pad_unit = std::max<int64_t>(itile, tile->jtile);

	std::vector<grav_univ_desc> univ(n_univ);
	int64_t body = 0, pad = 0, units = 0;
	for (int u = 0; u < n_univ; ++u) {
		if (n[u] < 0) return fail(GRAV_E_ARG, "n[%d] = %d < 0", u, n[u]);
		const int64_t nu = n[u];
		const int64_t npad = (nu + pad_unit - 1) / pad_unit * pad_unit;
		univ[u].body_off = body;
		univ[u].pad_off = pad;
		univ[u].n = static_cast<int32_t>(nu);
		univ[u].n_jtiles = static_cast<int32_t>((nu + tile->jtile - 1) / tile->jtile);
		univ[u].T = T ? T[u] : 0.0;
		body += nu;
		pad += npad;
		units += (npad / itile) * univ[u].n_jtiles;
	}
	const int64_t n_seg64 = pad / itile;
	if (n_seg64 > INT32_MAX) return fail(GRAV_E_ARG, "too many segments");
	const int32_t n_seg = static_cast<int32_t>(n_seg64);
	const int64_t grid = units > 0 ? std::min<int64_t>(tile->grid, units) : 0;

	std::vector<grav_seg_desc> seg(n_seg);
	int64_t unit = 0;
	int64_t slots = 0;
	int32_t s = 0;
	for (int u = 0; u < n_univ; ++u) {
		const int64_t npad = (u + 1 < n_univ ? univ[u + 1].pad_off : pad) - univ[u].pad_off;
		for (int64_t il = 0; il < npad; il += itile, ++s) {
			grav_seg_desc& d = seg[s];
			d.u = u;
			d.il0 = static_cast<int32_t>(il);
			d.unit_begin = unit;
			// i-tiles that hold only padding rows still exist (stage 2 zeroes them) but
			// have no work
			d.n_units = (il < univ[u].n) ? univ[u].n_jtiles : 0;
			if (d.n_units > 0) {
				// CTA c covers units [floor(c*U/G), floor((c+1)*U/G)); the CTA holding unit
				// x is ceil((x+1)*G/U) - 1
				const int64_t first = unit, last = unit + d.n_units - 1;
				const int64_t c0 = ((first + 1) * grid + units - 1) / units - 1;
				const int64_t c1 = ((last + 1) * grid + units - 1) / units - 1;
				d.cta_first = static_cast<int32_t>(c0);
				d.nslots = static_cast<int32_t>(c1 - c0 + 1);
				d.slot_base = static_cast<int32_t>(slots);
				slots += d.nslots;
			} else {
				d.cta_first = 0;
				d.nslots = 0;
				d.slot_base = static_cast<int32_t>(slots);
			}
			unit += d.n_units;
		}
	}
	if (slots > INT32_MAX) return fail(GRAV_E_ARG, "too many partial slots");

	info->n_bodies = body;
	info->n_pad_total = pad;
	info->n_units = units;
	info->n_univ = n_univ;
	info->n_seg = n_seg;
	info->n_slots = static_cast<int32_t>(slots);
	info->itile = static_cast<int32_t>(itile);
	info->pad_unit = static_cast<int32_t>(pad_unit);
	info->grid = static_cast<int32_t>(grid);
	if (univ_out && n_univ) std::memcpy(univ_out, univ.data(), sizeof(grav_univ_desc) * n_univ);
	if (seg_out && n_seg) std::memcpy(seg_out, seg.data(), sizeof(grav_seg_desc) * n_seg);
	return ok();
}

int grav_plan_pairs(int32_t n_univ, const int32_t* n, const double* T, const grav_tile* tile,
	grav_plan_info* info, grav_univ_desc* univ_out, grav_seg_desc* seg_out)
{
	if (n_univ < 0) return fail(GRAV_E_ARG, "n_univ < 0");
	if (n_univ > 0 && !n) return fail(GRAV_E_ARG, "n is NULL");
	if (!tile || !info) return fail(GRAV_E_ARG, "tile or info is NULL");
	if (tile->bpt <= 0 || tile->threads <= 0 || tile->jtile <= 0 || tile->grid <= 0)
		return fail(GRAV_E_ARG, "tile sizes must be positive");
	const auto pow2 = [](int x) { return x > 0 && (x & (x - 1)) == 0; };
	if (!pow2(tile->bpt) || !pow2(tile->threads) || !pow2(tile->jtile) || tile->threads < 32)
		return fail(GRAV_E_ARG, "tile sizes must be powers of two, threads >= 32");
	const int64_t R = static_cast<int64_t>(tile->bpt) * tile->threads;  // rows per block
	if (R % tile->jtile != 0) return fail(GRAV_E_ARG, "bpt*threads must be a multiple of jtile");
	const int64_t tpb = R / tile->jtile;

	std::vector<grav_univ_desc> univ(n_univ);
	int64_t body = 0, pad = 0, units = 0;
	for (int u = 0; u < n_univ; ++u) {
		if (n[u] < 0) return fail(GRAV_E_ARG, "n[%d] = %d < 0", u, n[u]);
		const int64_t nu = n[u];
		const int64_t nb = (nu + R - 1) / R;
		univ[u].body_off = body;
		univ[u].pad_off = pad;
		univ[u].n = static_cast<int32_t>(nu);
		univ[u].n_jtiles = static_cast<int32_t>((nu + tile->jtile - 1) / tile->jtile);
		univ[u].T = T ? T[u] : 0.0;
		for (int64_t I = 0; I < nb; ++I) units += univ[u].n_jtiles - I * tpb;
		body += nu;
		pad += nb * R;
	}
	const int64_t n_seg64 = pad / R;
	if (n_seg64 > INT32_MAX) return fail(GRAV_E_ARG, "too many segments");
	const int32_t n_seg = static_cast<int32_t>(n_seg64);
	const int64_t grid = units > 0 ? std::min<int64_t>(tile->grid, units) : 0;

	std::vector<grav_seg_desc> seg(n_seg);
	int64_t unit = 0, slots = 0;
	int32_t s = 0;
	for (int u = 0; u < n_univ; ++u) {
		const int64_t nb = (static_cast<int64_t>(univ[u].n) + R - 1) / R;
		for (int64_t I = 0; I < nb; ++I, ++s) {
			grav_seg_desc& d = seg[s];
			d.u = u;
			d.il0 = static_cast<int32_t>(I * R);
			d.unit_begin = unit;
			d.n_units = static_cast<int32_t>(univ[u].n_jtiles - I * tpb);
			const int64_t first = unit, last = unit + d.n_units - 1;
			const int64_t c0 = ((first + 1) * grid + units - 1) / units - 1;
			const int64_t c1 = ((last + 1) * grid + units - 1) / units - 1;
			d.cta_first = static_cast<int32_t>(c0);
			// row slots of the CTAs working on block I, then one column slot for each
			// block before it (written by the unique-pair tiles of those blocks)
			d.nslots = static_cast<int32_t>(c1 - c0 + 1 + I);
			d.slot_base = static_cast<int32_t>(slots);
			slots += d.nslots;
			unit += d.n_units;
		}
	}
	if (slots > INT32_MAX) return fail(GRAV_E_ARG, "too many partial slots");
	info->n_bodies = body;
	info->n_pad_total = pad;
	info->n_units = units;
	info->n_univ = n_univ;
	info->n_seg = n_seg;
	info->n_slots = static_cast<int32_t>(slots);
	info->itile = static_cast<int32_t>(R);
	info->pad_unit = static_cast<int32_t>(R);
	info->grid = static_cast<int32_t>(grid);
	if (univ_out && n_univ) std::memcpy(univ_out, univ.data(), sizeof(grav_univ_desc) * n_univ);
	if (seg_out && n_seg) std::memcpy(seg_out, seg.data(), sizeof(grav_seg_desc) * n_seg);
	return ok();
}

int64_t grav_pos_bytes(int mode, int64_t n_pad_total)
{
	if (!valid_mode(mode) || n_pad_total < 0) return fail(GRAV_E_ARG, "bad mode or size");
	if (mode == GRAV_MODE_FP64) return n_pad_total * 32;
	if (mode == GRAV_MODE_FP32C || mode == GRAV_MODE_FP32CU || mode == GRAV_MODE_FP32N ||
		mode == GRAV_MODE_FP32UN)
		return n_pad_total * 32;
	return n_pad_total * 16;
}

int64_t grav_part_bytes(const grav_plan_info* info)
{
	if (!info) return fail(GRAV_E_ARG, "info is NULL");
	return static_cast<int64_t>(info->n_slots) * 3 * info->itile * 8;
}

float grav_eps2(double max_gm)
{
	// keep eps2^-3/2 finite in FP32 (floor 1e-25 -> 3.2e37; the unique-pair kernel forms
	// rsqrt(r2)^3 before multiplying by the masses) and Gm * eps2^-3/2 <= 1e36 (FP32 max
	// is 3.4e38).  r2 + 1e-25 rounds to r2 for any separation above ~1.3e-9.
	double e = 1e-25;
	if (max_gm > 0.0) e = std::max(e, std::pow(max_gm / 1e36, 2.0 / 3.0));
	return static_cast<float>(e);
}

int grav_prepare(const grav_batch* b, void* stream)
{
	int rc = check_batch(b);
	if (rc) return rc;
	cudaError_t e = grav::launch_stage2(*b, GRAV_S2_PREPARE, static_cast<cudaStream_t>(stream));
	if (e != cudaSuccess) return cuda_fail(e, "stage-2 kernel launch (prepare)");
	return ok();
}

int grav_stage1(const grav_batch* b, void* stream)
{
	int rc = check_batch(b);
	if (rc) return rc;
	if (b->n_units == 0) return ok();
	if (!b->part || !b->err) return fail(GRAV_E_ARG, "NULL part or err pointer");
	if (b->tile.grid <= 0 || b->tile.grid > b->n_units)
		return fail(GRAV_E_ARG, "tile.grid (%d) must be in [1, n_units=%lld] (use grav_plan_info.grid)",
			b->tile.grid, (long long)b->n_units);
	const grav::Stage1Kernel* k = find_kernel(b->mode, b->tile.bpt, b->tile.threads, b->tile.jtile);
	if (!k)
		return fail(GRAV_E_TILE, "tile bpt=%d threads=%d jtile=%d not compiled for mode %d",
			b->tile.bpt, b->tile.threads, b->tile.jtile, b->mode);
	cudaError_t e = ensure_smem(k);
	if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute (dynamic shared memory)");
	grav_batch copy = *b;
	void* args[] = {&copy};
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	e = k->dependent
		? grav::launch_dependent(k->fn, b->tile.grid, b->tile.threads, k->smem_bytes, st, args)
		: cudaLaunchKernel(k->fn, dim3(b->tile.grid), dim3(b->tile.threads), args, k->smem_bytes, st);
	if (e != cudaSuccess) return cuda_fail(e, "stage-1 kernel launch");
	return ok();
}

int grav_stage2(const grav_batch* b, int flags, void* stream)
{
	int rc = check_batch(b);
	if (rc) return rc;
	if ((flags & ~(GRAV_S2_INTEGRATE | GRAV_S2_WRITE_A | GRAV_S2_PREPARE)) != 0)
		return fail(GRAV_E_ARG, "unknown stage-2 flags 0x%x", flags);
	if (!(flags & GRAV_S2_PREPARE)) {
		if (b->n_slots > 0 && !b->part) return fail(GRAV_E_ARG, "NULL part pointer");
		if ((flags & GRAV_S2_WRITE_A) && !b->a_out) return fail(GRAV_E_ARG, "NULL a_out pointer");
		if ((flags & GRAV_S2_INTEGRATE) && !b->v) return fail(GRAV_E_ARG, "NULL v pointer");
	}
	cudaError_t e = grav::launch_stage2(*b, flags, static_cast<cudaStream_t>(stream));
	if (e != cudaSuccess) return cuda_fail(e, "stage-2 kernel launch");
	return ok();
}

int grav_step(const grav_batch* b, int flags, void* stream)
{
	int rc = grav_stage1(b, stream);
	if (rc) return rc;
	return grav_stage2(b, flags & ~GRAV_S2_PREPARE, stream);
}

int grav_fused_supported(int mode, int32_t n, int32_t threads, int32_t rows)
{
	if (mode != GRAV_MODE_FP32 && mode != GRAV_MODE_FP32C && mode != GRAV_MODE_FP32N) return 0;
	if (n < 0 || n > GRAV_FUSED_MAX_N || rows < 1 || rows > threads) return 0;
	return grav::find_fused(mode, threads) != nullptr ? 1 : 0;
}

int grav_fused_occupancy(int mode, int32_t n, int32_t threads, int32_t rows,
	int32_t* ctas_per_sm)
{
	if (!ctas_per_sm) return fail(GRAV_E_ARG, "ctas_per_sm is NULL");
	if (!grav_fused_supported(mode, n, threads, rows))
		return fail(GRAV_E_TILE, "no single-launch step for mode %d, n %d, %d threads, %d rows",
			mode, n, threads, rows);
	int blocks = 0;
	if (grav::fused_occupancy(mode, n, threads, rows, &blocks) != 0)
		return fail(GRAV_E_CUDA, "occupancy query of the single-launch step failed");
	*ctas_per_sm = blocks;
	return ok();
}

int grav_step_fused(const grav_batch* b, int flags, int32_t threads, int32_t rows,
	int32_t* sync, void* stream)
{
	int rc = check_batch(b);
	if (rc) return rc;
	if (b->n_univ != 1) return fail(GRAV_E_ARG, "the single-launch step takes one universe (n_univ = %d)", b->n_univ);
	if (!sync) return fail(GRAV_E_ARG, "sync is NULL");
	if (flags & ~(GRAV_S2_INTEGRATE | GRAV_S2_WRITE_A))
		return fail(GRAV_E_ARG, "the single-launch step takes GRAV_S2_INTEGRATE and GRAV_S2_WRITE_A only");
	if ((flags & GRAV_S2_WRITE_A) && !b->a_out) return fail(GRAV_E_ARG, "GRAV_S2_WRITE_A without a_out");
	if (b->n_bodies > GRAV_FUSED_MAX_N)
		return fail(GRAV_E_SIZE, "%lld bodies: the single-launch step takes at most %d",
			(long long)b->n_bodies, GRAV_FUSED_MAX_N);
	if (!grav_fused_supported(b->mode, static_cast<int32_t>(b->n_bodies), threads, rows))
		return fail(GRAV_E_TILE, "no single-launch step for mode %d, %d threads, %d rows", b->mode,
			threads, rows);
	if (b->n_bodies == 0) return ok();
	cudaError_t e = grav::launch_fused(*b, flags, threads, rows, sync,
		static_cast<cudaStream_t>(stream));
	if (e != cudaSuccess) return cuda_fail(e, "single-launch step (cooperative launch)");
	return ok();
}

int grav_host_device_pointer(const void* host, void** dev)
{
	if (!host || !dev) return fail(GRAV_E_ARG, "NULL host or dev pointer");
	cudaPointerAttributes at;
	cudaError_t e = cudaPointerGetAttributes(&at, host);
	if (e != cudaSuccess) {
		cudaGetLastError();  // not a sticky error: clear it
		return fail(GRAV_E_ARG, "cudaPointerGetAttributes: %s", cudaGetErrorString(e));
	}
	if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr)
		return fail(GRAV_E_ARG, "%p is not page-locked host memory mapped for the device", host);
	*dev = at.devicePointer;
	return ok();
}

}  // extern "C"
