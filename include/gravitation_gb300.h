/*
 * gravitation_gb300.h -- C ABI of the GB300 all-pairs n-body engine (libgravgb300.so).
 *
 * The library is the stage-1/stage-2 hot path of one time step of the reference's
 * plugin API (gravitation/kernel/_base_.py:136-156): stage 1 computes
 *     a_i = sum_{j != i} G m_j (r_j - r_i) / |r_j - r_i|^3
 * and stage 2 applies the base class's symplectic Euler update
 *     v = a*T + v ;  r = v*T + r          (_base_.py:58-62)
 * on device memory owned by the caller.  Plain pointers and sizes only.
 *
 * Conventions
 *   - Every entry point returns 0 on success and a negative GRAV_E_* code on failure;
 *     grav_last_error() then describes the failure (thread-local string).
 *   - The library allocates no memory.  The caller owns every buffer; device buffers
 *     must stay valid until the work queued on `stream` has completed.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - Bodies are stored packed, universe after universe, as rows of 4 doubles:
 *       r[i] = (x, y, z, G*m)   and   v[i] = (vx, vy, vz, 0)
 *     with G already scaled as in _base_.py:85-88 and r, v, m scaled as in
 *     _base_.py:114-117.  The engine works on this FP64 state; stage 1 reads a padded
 *     copy of the positions (FP32 or FP64 by precision mode) that stage 2 refreshes.
 *   - Bodies at zero separation (the self pair and coincident distinct bodies) exert
 *     no force on each other.  The reference divides by zero there (np1.py:85-88).
 */
#ifndef GRAVITATION_GB300_H
#define GRAVITATION_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GRAV_ABI_VERSION 5

/* status codes */
#define GRAV_OK 0
#define GRAV_E_ARG -1         /* invalid argument (null pointer, bad size, bad mode) */
#define GRAV_E_TILE -2        /* tile shape not compiled into this library */
#define GRAV_E_CUDA -3        /* a CUDA runtime call failed */
#define GRAV_E_SIZE -4        /* caller buffer too small */
#define GRAV_E_DEVICE -5      /* device is not a GB300-class (sm_103) GPU */

/* device error flag values written by kernels into grav_batch.err */
#define GRAV_DEV_OK 0
#define GRAV_DEV_TIMEOUT 1    /* a bounded device wait expired (bulk copy, grid barrier) */

/* precision modes (universe_base dtype / kernel meta "precision") */
#define GRAV_MODE_FP32 0      /* FP32 separations and weights, compensated FP32 (hi + lo) sums */
#define GRAV_MODE_FP32C 1     /* as FP32 with double-single (hi+lo) positions: separations exact */
#define GRAV_MODE_FP64 2      /* FP64 throughout */
#define GRAV_MODE_FP32U 3     /* FP32 arithmetic of GRAV_MODE_FP32 on unique pairs (each pair
                                 once, both bodies updated); plan with grav_plan_pairs */
#define GRAV_MODE_FP32CU 4    /* GRAV_MODE_FP32C's double-single positions on unique pairs;
                                 plan with grav_plan_pairs */
#define GRAV_MODE_FP32N 5     /* GRAV_MODE_FP32 with near pairs corrected: every pair closer
                                 than max|x_i| / GRAV_NEAR_KAPPA (max over the coordinates of
                                 the rows a thread holds) is evaluated from the double-single
                                 separation (hi_j - hi_i) + (lo_j - lo_i) instead of the FP32
                                 one; a pair whose FP32 separation is exactly zero contributes
                                 nothing, as in GRAV_MODE_FP32 */
#define GRAV_MODE_FP32UN 6    /* GRAV_MODE_FP32N's correction on unique pairs; plan with
                                 grav_plan_pairs */

/* Near-pair radius of GRAV_MODE_FP32N / GRAV_MODE_FP32UN in units of the coordinate
 * magnitude: beyond |x| / 20 the FP32 rounding of the positions changes a pair term by
 * at most ~4.5e-6 of itself. */
#define GRAV_NEAR_KAPPA 20

/* stage-2 flags */
#define GRAV_S2_INTEGRATE 1   /* v = a*T + v ; r = v*T + r */
#define GRAV_S2_WRITE_A 2     /* write the accelerations to a_out */
#define GRAV_S2_PREPARE 4     /* only refresh the padded stage-1 positions from r */

/* One universe of a packed batch (device array, built by grav_plan). */
typedef struct grav_univ_desc {
	int64_t body_off;  /* first row of this universe in r, v, a_out */
	int64_t pad_off;   /* first row in the padded stage-1 position array */
	int32_t n;         /* number of bodies */
	int32_t n_jtiles;  /* ceil(n / jtile) */
	double T;          /* time step of this universe */
} grav_univ_desc;

/* One i-tile of one universe: the unit of the persistent work list (device array). */
typedef struct grav_seg_desc {
	int64_t unit_begin; /* index of its first work unit (one j-tile) in the global order */
	int32_t u;          /* universe */
	int32_t il0;        /* first local body of the i-tile */
	int32_t n_units;    /* j-tiles to visit (0 for a tile made only of padding) */
	int32_t cta_first;  /* first CTA of the persistent grid that works on it */
	int32_t slot_base;  /* first partial-sum slot of this segment */
	int32_t nslots;     /* its slots: one per CTA that works on it (+ column slots, pair plans) */
} grav_seg_desc;

/* Tile shape of the stage-1 kernel. */
typedef struct grav_tile {
	int32_t bpt;      /* i-bodies held in registers per thread */
	int32_t threads;  /* threads per CTA */
	int32_t jtile;    /* j-bodies per shared-memory tile (one bulk copy) */
	int32_t grid;     /* persistent CTAs (clamped to the number of work units) */
} grav_tile;

/* Sizes derived by grav_plan. */
typedef struct grav_plan_info {
	int64_t n_bodies;    /* sum of n over universes (rows of r, v, a_out) */
	int64_t n_pad_total; /* rows of the padded stage-1 position array */
	int64_t n_units;     /* total work units (i-tile x j-tile) */
	int32_t n_univ;
	int32_t n_seg;       /* = n_pad_total / itile */
	int32_t n_slots;     /* partial-sum slots (each 3 x itile 8-byte entries) */
	int32_t itile;       /* bpt * threads */
	int32_t pad_unit;    /* max(itile, jtile) */
	int32_t grid;        /* CTAs actually launched */
} grav_plan_info;

/* Everything one stage-1/stage-2 launch needs.  All pointers are device pointers. */
typedef struct grav_batch {
	int32_t mode;                 /* GRAV_MODE_* */
	int32_t n_univ;
	int32_t n_seg;
	int32_t n_slots;
	int64_t n_bodies;
	int64_t n_pad_total;
	int64_t n_units;
	grav_tile tile;               /* tile.grid = CTAs launched (grav_plan_info.grid) */
	float eps2;                   /* r^2 floor for the FP32 modes (see grav_eps2) */
	float _pad0;
	const grav_univ_desc* univ;   /* n_univ */
	const grav_seg_desc* seg;     /* n_seg */
	double* r;                    /* n_bodies x 4 */
	double* v;                    /* n_bodies x 4 */
	void* pos;                    /* padded stage-1 positions, grav_pos_bytes() */
	double* part;                 /* n_slots x 3 x itile (scratch of stage 1 -> stage 2) */
	double* a_out;                /* n_bodies x 4, may be NULL unless GRAV_S2_WRITE_A */
	int32_t* err;                 /* one device int, GRAV_DEV_* (first error wins) */
} grav_batch;

/* ---- library ---------------------------------------------------------------- */

/* ABI version (GRAV_ABI_VERSION).  No reference counterpart. */
int grav_abi_version(void);

/* Message describing the last failure on this thread (never NULL). */
const char* grav_last_error(void);

/* SM count and compute capability of `device`.  Fails with GRAV_E_DEVICE on a GPU
 * other than compute capability 10.3 (the library holds sm_103a code only). */
int grav_device_query(int device, int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);

/* 1 if the tile shape is compiled for `mode`, else 0. */
int grav_tile_supported(int mode, const grav_tile* tile);

/* Number of compiled tile shapes for `mode`; fills up to `cap` entries of `out`. */
int grav_tile_list(int mode, grav_tile* out, int cap);

/* Resident CTAs per SM of the stage-1 kernel for `mode` and `tile` on the current
 * device (the persistent grid is sm_count * this). */
int grav_occupancy(int mode, const grav_tile* tile, int32_t* ctas_per_sm);

/* ---- planning (host only, no GPU needed) ------------------------------------- */

/*
 * Lay out `n_univ` universes of sizes n[u] (time steps T[u]) for the persistent
 * stage-1 kernel with the given tile.  Two-call protocol: call with univ_out and
 * seg_out NULL to fill `info`, then again with arrays of info->n_univ and
 * info->n_seg entries.  The tables must then be copied to device memory.
 * Replaces the reference's per-kernel set-up in start_kernel (e.g. np2.py:57-87,
 * pc2.py:99-145); the work list has no reference counterpart.
 */
int grav_plan(int32_t n_univ, const int32_t* n, const double* T, const grav_tile* tile,
	grav_plan_info* info, grav_univ_desc* univ_out, grav_seg_desc* seg_out);

/*
 * Plan for GRAV_MODE_FP32U (same protocol and outputs as grav_plan).  Universes are cut
 * into row blocks of bpt*threads bodies (segments); the units of block I are the
 * j-tiles of blocks J >= I.  Segment J's slots are its row slots followed by one column
 * slot per block I < J.  Requires threads >= 32 and bpt*threads a multiple of jtile.
 * Replaces the unique-pair row partition of the reference's CPU kernels
 * (np1.py:104-105, _lib1_/lib.c:70-124, _lib4_/lib.c:76-144).
 */
int grav_plan_pairs(int32_t n_univ, const int32_t* n, const double* T, const grav_tile* tile,
	grav_plan_info* info, grav_univ_desc* univ_out, grav_seg_desc* seg_out);

/* Bytes of the padded stage-1 position array for `mode` and `n_pad_total` rows. */
int64_t grav_pos_bytes(int mode, int64_t n_pad_total);

/* Bytes of the partial-sum buffer (grav_batch.part) for a plan: 3 x itile 8-byte entries
 * per slot. */
int64_t grav_part_bytes(const grav_plan_info* info);

/* r^2 floor for the FP32 modes: max(1e-25, (max_gm / 1e36)^(2/3)), the smallest value
 * that keeps both r^-3 and G*m * r^-3 finite in FP32 at zero separation.  r^2 + eps2
 * rounds to r^2 for any separation above ~1.3e-9 (for max_gm <= 0.03), far below the
 * FP32 resolution of the coordinates of any realistic universe, so it does not act as
 * softening: it only makes zero-separation terms vanish (their d is exactly 0). */
float grav_eps2(double max_gm);

/* ---- stages (device work, asynchronous on `stream`) ---------------------------- */

/* Refresh the padded stage-1 positions from r (after r was written by the host). */
int grav_prepare(const grav_batch* b, void* stream);

/*
 * Stage 1: partial sums of the accelerations into b->part (FP32 (hi, lo) compensated
 * pairs per row and FP32 column sums in the FP32 modes, FP64 values in GRAV_MODE_FP64).
 * Replaces universe_base.step_stage1 (_base_.py:147-150) as realised by
 * np1.update_pair/step_stage1 (np1.py:81-108), c1a's step_stage1
 * (_lib1_/lib.c:52-126) and pc2.update_all (pc2.py:59-91).
 */
int grav_stage1(const grav_batch* b, void* stream);

/*
 * Stage 2: sum the partials (compensated FP32 in the FP32 modes, widened to FP64 once per
 * body; FP64 in GRAV_MODE_FP64), optionally write a_out, optionally integrate
 * (v = a*T + v; r = v*T + r in FP64, no fused multiply-add, as _base_.py:58-62 and
 * np2.py:110-115), then refresh the padded stage-1 positions.
 * Replaces universe_base.step_stage2 (_base_.py:152-156) / np2.step_stage2.
 */
int grav_stage2(const grav_batch* b, int flags, void* stream);

/* Stage 1 then stage 2 with `flags` (one full step when GRAV_S2_INTEGRATE).
 * Replaces universe_base.step's stage 1 and stage 2 calls (_base_.py:143-144). */
int grav_step(const grav_batch* b, int flags, void* stream);

/* ---- single-launch step for one small universe ---------------------------------- */

/* Largest universe grav_step_fused takes (every CTA holds all positions in shared
 * memory). */
#define GRAV_FUSED_MAX_N 4096

/* 1 if grav_step_fused has a kernel for `mode` (GRAV_MODE_FP32, GRAV_MODE_FP32C or
 * GRAV_MODE_FP32N), `threads` per CTA (256, 512 or 1024) and `rows` per CTA
 * (1 <= rows <= threads) at n bodies (n <= GRAV_FUSED_MAX_N), else 0. */
int grav_fused_supported(int mode, int32_t n, int32_t threads, int32_t rows);

/* Resident CTAs per SM of that kernel on the current device; grav_step_fused launches
 * ceil(n / rows) CTAs, which must not exceed SMs x this. */
int grav_fused_occupancy(int mode, int32_t n, int32_t threads, int32_t rows,
	int32_t* ctas_per_sm);

/*
 * One full step (GRAV_S2_INTEGRATE, optionally GRAV_S2_WRITE_A) of a batch holding one
 * universe (laid out by grav_plan: its rows start at row 0 of r, v and pos, and
 * b->n_bodies is its size), in a single launch of ceil(n / rows) CTAs of `threads`
 * threads (one thread-block cluster up to 16 CTAs where the GPU can schedule it, else a
 * cooperative launch).  Each CTA copies every body's stage-1 position to shared memory,
 * completes the accelerations of its `rows` rows over all bodies and applies stage 2 to
 * them: the same pair arithmetic, compensated sums and FP64 update as grav_stage1 +
 * grav_stage2, summed in another order (results agree to FP32 rounding of the partial
 * sums).  The writes wait for every CTA's copy: on the cluster barrier, or on a grid
 * barrier over `sync`, two device int32 that are zero before the first call and that
 * every completed call leaves zero.  The grid barrier's wait is bounded: after 2 s it
 * sets GRAV_DEV_TIMEOUT in b->err and the step writes nothing (zero `sync` again before
 * the next call).  b->part is not used.  Replaces universe_base.step's stage 1 and
 * stage 2 calls (_base_.py:143-144) for universes of up to GRAV_FUSED_MAX_N bodies,
 * where launch latency sets the step's time.
 */
int grav_step_fused(const grav_batch* b, int flags, int32_t threads, int32_t rows,
	int32_t* sync, void* stream);

/* ---- diagnostics -------------------------------------------------------------------- */

/*
 * Energy and momentum of every universe in FP64.  `b` is an FP64 view of the batch:
 * mode GRAV_MODE_FP64, pos = padded double4 positions refreshed by grav_prepare on that
 * view, part = scratch of grav_part_bytes() (overwritten).  out: n_univ x 8 doubles
 * (device), per universe
 *   [0] sum 1/2 Gm v^2   [1] -1/2 sum_i Gm_i sum_{j!=i} Gm_j / |r_j - r_i|
 *   [2..4] sum Gm v      [5..7] 0
 * (divide by G for kinetic energy, potential energy and momentum).  Reduction order is
 * fixed, so results are reproducible.  No reference counterpart (an accuracy analysis
 * is a wish in the reference, TODO.md:4).
 */
int grav_energy(const grav_batch* b, double* out, void* stream);

/* ---- adjoint (reverse-mode gradients) -------------------------------------------------- */

/* Buffers of the backward sweep.  `b` is a batch planned with an adjoint tile
 * (grav_adjoint_tile_supported): mode GRAV_MODE_FP32 with grav_plan (every ordered pair)
 * or GRAV_MODE_FP32U with grav_plan_pairs (each unordered pair once); b->r, b->v hold
 * the state being reversed (start: the state after the last forward step of the
 * segment), b->pos is scratch. */
typedef struct grav_adjoint {
	const grav_batch* b;
	double* gr;    /* n_bodies x 4: dL/dr of the current state (in/out) */
	double* gv;    /* n_bodies x 4: dL/dv of the current state (in/out) */
	double* ggm;   /* n_bodies: dL/d(G m), accumulated (in/out) */
	void* upos;    /* float4 [n_pad_total]: scratch, FP32 u = gv + T gr of the next step */
	double* part7; /* n_slots x 7 x itile doubles: scratch */
	const double* a_in; /* n_bodies x 4: the forward's accelerations a_k of the step being
	                       reversed (as stage 2 wrote them with GRAV_S2_WRITE_A), or NULL:
	                       the pair kernel then recomputes them */
} grav_adjoint;

/* 1 if `tile` has a compiled adjoint pair kernel for `mode` (GRAV_MODE_FP32: all
 * ordered pairs; GRAV_MODE_FP32U: unique pairs). */
int grav_adjoint_tile_supported(int mode, const grav_tile* tile);

/* Resident CTAs per SM of the adjoint pair kernel for `mode` and `tile` on the current
 * device. */
int grav_adjoint_occupancy(int mode, const grav_tile* tile, int32_t* ctas_per_sm);

/* Start of a backward segment: from b->r, b->v (state k+1) and gr, gv, write the FP32
 * positions r_k = r_{k+1} - T v_{k+1} and u = gv + T gr used by the next step. */
int grav_adjoint_prepare(const grav_adjoint* a, void* stream);

/*
 * One backward step through stage 2 and stage 1 (the adjoint kernel pair): a pair
 * kernel forms h = J_A(r_k)^T u and g_j = sum_i u_i.(r_i - r_j)/|r_i - r_j|^3, and
 * recomputes a_k = A(r_k) (stage 1) unless a->a_in holds it; the adjoint stage 2
 * reverses the state (r_k = r_{k+1} - T v_{k+1}, v_k = v_{k+1} - T a_k, FP64), updates
 * gr += T h, gv = u, ggm -= T g, and prepares the next step.
 * Transposes universe_base.step_stage1/step_stage2 (_base_.py:147-156); no
 * counterpart in the reference (it has no gradients).
 */
int grav_adjoint_step(const grav_adjoint* a, void* stream);

/* ---- allocation-free variant ------------------------------------------------------- */

/* Largest universe grav_forces_noalloc accepts. */
#define GRAV_NOALLOC_MAX_N 16384

/*
 * Accelerations of one universe of n <= GRAV_NOALLOC_MAX_N bodies for callers that
 * cannot allocate device memory where they need forces (code inside another
 * framework's memory pool, threads that must not enter the CUDA allocator while other
 * work is captured or timed, hosts that reserve all device memory up front).
 * Inputs: r, n x 4 doubles (x, y, z, G*m) on the device; max_gm = the largest G*m
 * (sets the FP32 r^2 floor, see grav_eps2).  Output: a, n x 4 doubles (ax, ay, az, 0).
 * err: optional device int that the kernels set to a GRAV_DEV_* code when a bounded
 * wait expires (first error wins); the call never clears it, so the caller zeroes it
 * before the first call and may share it with other work.  With err = NULL the kernels
 * use an internal flag that no caller can read: a device-side timeout then goes
 * unreported (the accelerations of that call are incomplete), so pass a flag wherever
 * that matters.
 * Same arithmetic as grav_stage1 + grav_stage2(GRAV_S2_WRITE_A) in GRAV_MODE_FP32, on a
 * fixed tile (2 bodies/thread, 128 threads, 128-body j-tiles).
 * It calls no cudaMalloc/cudaFree or other allocating routine: its scratch (plan
 * tables, padded positions, FP32 (hi, lo) partial sums, error flag) is one file-scope
 * device array of about 3.8 MB that every GPU loading the library holds until exit.  The first
 * call on each device, with that device current, looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  Every call
 * shares the array: calls whose work overlaps on the GPU race.  n above the limit is
 * rejected with GRAV_E_SIZE.  Failures are described by grav_last_error().
 * No counterpart in the reference.
 */
int grav_forces_noalloc(const double* r, double* a, int32_t n, double max_gm, int32_t* err,
	void* stream);

/* ---- scenarios generated on the device ---------------------------------------------- */

/* Scenario kinds (grav_scenario.kind). */
#define GRAV_SCEN_UNIFORM_CUBE 1 /* p = {half, v_sigma, m_lo, m_hi} */
#define GRAV_SCEN_PLUMMER 2      /* p = {a, m_lo, m_hi, cx, cy, cz, cvx, cvy, cvz} */
#define GRAV_SCEN_GALAXY 3       /* p = {radius, m_hole, m_star, scale_r, scale_m} */

/*
 * A seeded scenario.  Random numbers come from the counter-based Philox4x64-10
 * generator (Salmon, Moraes, Dror, Shaw, SC'11): key = {seed, stream}, counter =
 * {body index, block, 0, 0}, so every body draws independently of the others and the
 * result does not depend on the launch shape.  A uniform double is
 * (word >> 11) * 2^-53, as numpy's generators convert 64-bit words.
 *
 *  UNIFORM_CUBE  r ~ U[-half, half]^3, v ~ N(0, v_sigma^2)^3 (Box-Muller),
 *                m ~ U[m_lo, m_hi]: the bench configurations' bodies.
 *  PLUMMER       one Plummer sphere of scale radius a (Aarseth, Henon & Wielen 1974:
 *                radius from the inverted cumulative mass cut at 99.9 %, isotropic
 *                directions, speed q * v_esc with q drawn by rejection from
 *                q^2 (1 - q^2)^(7/2)), masses log-uniform in [m_lo, m_hi], then shifted
 *                so that its centre of mass sits at (cx, cy, cz) moving with
 *                (cvx, cvy, cvz).  Two calls with different streams and offsets into
 *                r/v make the colliding pair.
 *  GALAXY        the reference's galaxy recipe (simulation.py:99-184): a central mass
 *                m_hole at the origin and n - 1 stars of m_star on circular orbits about
 *                it, the first 4/5 in a thin disc, the rest in a bulge; SI inputs are
 *                scaled by scale_r / scale_m as add_object does (_base_.py:114-117) and
 *                G is the universe's scaled G (_base_.py:85-88), used for the orbital
 *                speeds as the recipe does (simulation.py:147-149).
 *
 * Output: r (x, y, z, G*m) and v (vx, vy, vz, 0), n rows of 4 doubles each, the packed
 * layout of grav_batch (pass r + 4 * body_off for a universe inside a batch).
 */
typedef struct grav_scenario {
	int32_t kind;
	int32_t _pad0;
	uint64_t seed;
	uint64_t stream;
	double G;     /* column 3 of r receives G * m */
	double p[10]; /* kind parameters, see GRAV_SCEN_* */
} grav_scenario;

/* Device scratch grav_scenario_generate needs for n bodies of this kind (0: none). */
int64_t grav_scenario_scratch_bytes(const grav_scenario* s, int64_t n);

/*
 * Writes n bodies of scenario s into the device (or device-addressable) arrays r and v
 * (32-byte aligned).  scratch: grav_scenario_scratch_bytes() bytes of device memory
 * (NULL when that is 0).  Deterministic: the same s and n give the same bits on every
 * call.  Replaces the reference's Python generators + add_object loop
 * (simulation.py:85-184, _base_.py:107-118) for the bodies' initial state.
 */
int grav_scenario_generate(const grav_scenario* s, double* r, double* v, int64_t n,
	void* scratch, void* stream);

/* ---- host-resident state ------------------------------------------------------------ */

/*
 * Device address of page-locked host memory (cudaHostAlloc / cudaHostRegister, e.g. a
 * pinned PyTorch tensor).  A grav_batch whose r and v point there makes grav_prepare
 * and grav_stage2 read and write the host copy in place over the CPU-GPU link, so a
 * host-synchronised step needs no separate copies.  Writes *dev, or returns GRAV_E_ARG
 * when `host` is not page-locked memory that the current device can address.
 * No counterpart in the reference (its kernels copy numpy arrays in and out every
 * step, np1.py:101-108, pc2.py:147-168).
 */
int grav_host_device_pointer(const void* host, void** dev);

/* ---- failure path check -------------------------------------------------------------- */

/* Test hook: one CTA waits, with the library's bounded wait and a limit of `limit_ns`
 * (<= 2e9), on an mbarrier that nothing completes, then writes GRAV_DEV_TIMEOUT to the
 * device int `err` and returns.  Shows that an expired wait is reported to the host and
 * leaves the context usable.  No reference counterpart. */
int grav_wait_check(int32_t* err, int64_t limit_ns, void* stream);

/* ---- measurement ------------------------------------------------------------------ */

/* FP32 FMA throughput probe: `blocks` CTAs of 256 threads, each thread 8 independent
 * FMA chains of 16*iters FMAs; writes blocks*256 floats to `out`.  Timed by the caller,
 * it gives the FP32 peak (2 FLOP per FMA) the stage-1 roofline is quoted against.
 * No reference counterpart (the reference times wall clock only, lib/timing.py:41-78). */
int grav_fp32_peak_probe(float* out, int32_t blocks, int32_t iters, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GRAVITATION_GB300_H */
