// noalloc.cu -- accelerations of one universe without allocating any memory.
//
// Some callers cannot allocate device memory at the point where they need forces:
// code running inside another framework's memory pool with no allocation hook, a
// host thread that must not enter the CUDA allocator while other work is being
// captured or timed, or embedded hosts that reserve all device memory up front.
// grav_forces_noalloc serves them: the caller passes only the inputs (positions and
// G*m) and the output (accelerations); every piece of scratch memory the stage-1 and
// stage-2 kernels need -- plan tables, padded FP32 positions, FP32 (hi, lo) partial
// sums and the device error flag -- lives in the file-scope array below, sized for at most
// GRAV_NOALLOC_MAX_N bodies (about 3.8 MB, held by every GPU that loads the library
// until the process exits).
//
// Host code never dereferences g_noalloc_scratch: in host code that name is only a
// host-side stand-in for the device symbol.  The first call on each device (with that
// device current) asks the runtime for the array's device address with
// cudaGetSymbolAddress and keeps it; that first call should come before any stream
// capture.  All calls share the array and it keeps the last call's contents: each
// call rebuilds the plan tables, rewrites all the padded positions and partial slots it
// reads and zeroes the internal error flag, so nothing stale is read, but two calls whose
// work overlaps on the GPU (different streams, no ordering between them) race on it.
// A caller-supplied error flag is never cleared here (the caller owns it and may share
// it); with none, device-side timeouts land in the internal flag and go unreported.
#include <cstdio>
#include <mutex>

#include "grav_types.h"

namespace grav {
// sets the message grav_last_error() returns (abi.cu); only failure paths call it
int record_error(int code, const char* msg);
}

extern "C" int grav_stage1(const grav_batch* b, void* stream);
extern "C" int grav_stage2(const grav_batch* b, int flags, void* stream);

namespace {

// fixed tile of the FP32 stage-1 kernel used here (compiled in stage1_f32.cu)
constexpr int NA_BPT = 2, NA_THREADS = 128, NA_JTILE = 128;
constexpr int NA_ITILE = NA_BPT * NA_THREADS;                           // 256
constexpr int NA_PAD = NA_ITILE > NA_JTILE ? NA_ITILE : NA_JTILE;       // 256
constexpr int NA_MAX_SEG = GRAV_NOALLOC_MAX_N / NA_PAD;                 // 64
constexpr int NA_MAX_GRID = 512;
constexpr int NA_MAX_SLOTS = NA_MAX_SEG + NA_MAX_GRID;
constexpr int NA_MAX_DEVICES = 64;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t OFF_UNIV = 0;
constexpr size_t OFF_SEG = align256(OFF_UNIV + sizeof(grav_univ_desc));
constexpr size_t OFF_ERR = align256(OFF_SEG + NA_MAX_SEG * sizeof(grav_seg_desc));
constexpr size_t OFF_POS = align256(OFF_ERR + sizeof(int32_t));
constexpr size_t OFF_PART = align256(OFF_POS + size_t(GRAV_NOALLOC_MAX_N) * 16);
constexpr size_t SCRATCH_BYTES = align256(OFF_PART + size_t(NA_MAX_SLOTS) * 3 * NA_ITILE * 8);

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

struct DeviceSetup {
	bool done;
	unsigned char* scratch;  // device address of g_noalloc_scratch on this device
	int grid_cap;            // SMs x resident CTAs of the stage-1 kernel, <= NA_MAX_GRID
};
DeviceSetup g_setup[NA_MAX_DEVICES];
std::mutex g_setup_mutex;

int na_fail(int code, const char* fmt, long long value)
{
	char msg[256];
	snprintf(msg, sizeof(msg), fmt, value);
	return grav::record_error(code, msg);
}

// The single-universe plan of grav_plan, without any container: segment s covers
// bodies [s*NA_ITILE, (s+1)*NA_ITILE); CTA c of `grid` takes units
// [c*units/grid, (c+1)*units/grid).  Writes the tables when `seg` is non-null and
// returns the number of partial-sum slots.
__host__ __device__ int plan_single(int n, int grid, long long units, grav_seg_desc* seg)
{
	const int n_pad = (n + NA_PAD - 1) / NA_PAD * NA_PAD;
	const int n_seg = n_pad / NA_ITILE;
	const int nj = (n + NA_JTILE - 1) / NA_JTILE;
	long long unit = 0;
	int slots = 0;
	for (int s = 0; s < n_seg; ++s) {
		const int il0 = s * NA_ITILE;
		const int n_units = il0 < n ? nj : 0;
		int c0 = 0, ns = 0;
		if (n_units > 0) {
			const long long first = unit, last = unit + n_units - 1;
			c0 = static_cast<int>(((first + 1) * grid + units - 1) / units - 1);
			const int c1 = static_cast<int>(((last + 1) * grid + units - 1) / units - 1);
			ns = c1 - c0 + 1;
		}
		if (seg) {
			seg[s].unit_begin = unit;
			seg[s].u = 0;
			seg[s].il0 = il0;
			seg[s].n_units = n_units;
			seg[s].cta_first = c0;
			seg[s].slot_base = slots;
			seg[s].nslots = ns;
		}
		slots += ns;
		unit += n_units;
	}
	return slots;
}

// Writes the plan tables and clears the internal error flag (a caller's flag is left
// alone).  The launches after it read the tables, so the next one (the prepare pass) is
// launched the ordinary way: it starts only after this kernel has completed.
__global__ void noalloc_plan_kernel(unsigned char* scratch, int n, int grid, long long units)
{
	if (blockIdx.x != 0 || threadIdx.x != 0) return;
	grav_univ_desc* u = reinterpret_cast<grav_univ_desc*>(scratch + OFF_UNIV);
	u->body_off = 0;
	u->pad_off = 0;
	u->n = n;
	u->n_jtiles = (n + NA_JTILE - 1) / NA_JTILE;
	u->T = 0.0;
	plan_single(n, grid, units, reinterpret_cast<grav_seg_desc*>(scratch + OFF_SEG));
	*reinterpret_cast<int32_t*>(scratch + OFF_ERR) = GRAV_DEV_OK;
}

int device_setup(DeviceSetup** out)
{
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return na_fail(GRAV_E_CUDA, "cudaGetDevice failed (%lld)", (long long)e);
	if (dev < 0 || dev >= NA_MAX_DEVICES)
		return na_fail(GRAV_E_DEVICE, "device ordinal %lld out of range", (long long)dev);
	std::lock_guard<std::mutex> lock(g_setup_mutex);
	DeviceSetup& s = g_setup[dev];
	if (!s.done) {
		void* p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess || !p)
			return na_fail(GRAV_E_CUDA, "cudaGetSymbolAddress of the scratch array failed (%lld)",
				(long long)e);
		int sms = 0;
		e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		if (e != cudaSuccess) return na_fail(GRAV_E_CUDA, "SM count query failed (%lld)", (long long)e);
		const grav::Stage1Kernel* tab = nullptr;
		const int nk = grav::stage1_table_f32(&tab);
		const grav::Stage1Kernel* k = nullptr;
		for (int i = 0; i < nk; ++i)
			if (tab[i].mode == GRAV_MODE_FP32 && tab[i].bpt == NA_BPT &&
				tab[i].threads == NA_THREADS && tab[i].jtile == NA_JTILE)
				k = &tab[i];
		if (!k) return na_fail(GRAV_E_TILE, "fixed tile %lld not compiled", (long long)NA_ITILE);
		int occ = 0;
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k->fn, NA_THREADS, k->smem_bytes);
		if (e != cudaSuccess || occ <= 0)
			return na_fail(GRAV_E_CUDA, "occupancy query failed (%lld)", (long long)e);
		s.scratch = static_cast<unsigned char*>(p);
		s.grid_cap = sms * occ < NA_MAX_GRID ? sms * occ : NA_MAX_GRID;
		s.done = true;
	}
	*out = &s;
	return GRAV_OK;
}

}  // namespace

extern "C" int grav_forces_noalloc(const double* r, double* a, int32_t n, double max_gm,
	int32_t* err, void* stream)
{
	if (n < 0) return na_fail(GRAV_E_ARG, "n = %lld < 0", (long long)n);
	if (n > GRAV_NOALLOC_MAX_N)
		return na_fail(GRAV_E_SIZE, "n = %lld exceeds the no-allocation limit of "
			"GRAV_NOALLOC_MAX_N = 16384 bodies", (long long)n);
	if (n == 0) return GRAV_OK;
	if (!r || !a) return grav::record_error(GRAV_E_ARG, "NULL r or a pointer");
	if (!(max_gm >= 0.0)) return grav::record_error(GRAV_E_ARG, "max_gm must be >= 0");

	DeviceSetup* s = nullptr;
	int rc = device_setup(&s);
	if (rc) return rc;
	cudaStream_t st = static_cast<cudaStream_t>(stream);

	const int n_pad = (n + NA_PAD - 1) / NA_PAD * NA_PAD;
	const long long units = static_cast<long long>((n + NA_ITILE - 1) / NA_ITILE) *
		((n + NA_JTILE - 1) / NA_JTILE);
	const int grid = static_cast<int>(units < s->grid_cap ? units : s->grid_cap);
	const int n_slots = plan_single(n, grid, units, nullptr);
	int32_t* errp = err ? err : reinterpret_cast<int32_t*>(s->scratch + OFF_ERR);

	noalloc_plan_kernel<<<1, 32, 0, st>>>(s->scratch, n, grid, units);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return na_fail(GRAV_E_CUDA, "plan kernel launch failed (%lld)", (long long)e);

	grav_batch b = {};
	b.mode = GRAV_MODE_FP32;
	b.n_univ = 1;
	b.n_seg = n_pad / NA_ITILE;
	b.n_slots = n_slots;
	b.n_bodies = n;
	b.n_pad_total = n_pad;
	b.n_units = units;
	b.tile = grav_tile{NA_BPT, NA_THREADS, NA_JTILE, grid};
	b.eps2 = grav_eps2(max_gm);
	b.univ = reinterpret_cast<const grav_univ_desc*>(s->scratch + OFF_UNIV);
	b.seg = reinterpret_cast<const grav_seg_desc*>(s->scratch + OFF_SEG);
	b.r = const_cast<double*>(r);  // read only: no GRAV_S2_INTEGRATE below
	b.v = nullptr;
	b.pos = s->scratch + OFF_POS;
	b.part = reinterpret_cast<double*>(s->scratch + OFF_PART);
	b.a_out = a;
	b.err = errp;
	// the prepare pass reads the tables the plan kernel just wrote before its
	// grid_dep_wait(), so it must not start early: an ordinary launch
	e = grav::launch_stage2(b, GRAV_S2_PREPARE, st, false);
	if (e != cudaSuccess)
		return na_fail(GRAV_E_CUDA, "prepare kernel launch failed (%lld)", (long long)e);
	if ((rc = grav_stage1(&b, st)) != GRAV_OK) return rc;
	return grav_stage2(&b, GRAV_S2_WRITE_A, st);
}
