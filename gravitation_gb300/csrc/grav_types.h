// grav_types.h -- internal constants shared by host and device code of libgravgb300.
#pragma once

#include <cuda_runtime.h>

#include "gravitation_gb300.h"

// Wall-clock bound of every device-side wait on a bulk copy (nanoseconds).
#define GRAV_WAIT_NS 2000000000ull

namespace grav {

// Launch-time view of one stage-1 kernel instantiation.
struct Stage1Kernel {
	int mode, bpt, threads, jtile;
	const void* fn;       // __global__ function
	int smem_bytes;       // dynamic shared memory per CTA
	bool dependent;       // waits with grid_dep_wait(): may launch as a programmatic dependent
};

// Stage-2 kernel (stage2.cu).  dependent = true launches it with programmatic stream
// serialization (it reads only plan tables before its grid_dep_wait()); false launches
// it the ordinary way, for callers whose previous kernel wrote those tables.
cudaError_t launch_stage2(const grav_batch& b, int flags, cudaStream_t stream,
	bool dependent = true);

// Single-launch step of one small universe (fused.cu).
const void* find_fused(int mode, int threads);
cudaError_t launch_fused(const grav_batch& b, int flags, int threads, int rows, int32_t* sync,
	cudaStream_t stream);
int fused_occupancy(int mode, int64_t n, int threads, int rows, int* ctas_per_sm);

// Kernel tables, one per translation unit (stage1_f32.cu, stage1_f64.cu).
int stage1_table_f32(const Stage1Kernel** out);
int stage1_table_f64(const Stage1Kernel** out);
int stage1_table_sym(const Stage1Kernel** out);

// Launch with programmatic stream serialization: the kernel may begin while the kernel
// before it in the stream finishes; it must call grid_dep_wait() (grav_device.cuh)
// before touching anything that kernel, or one before it, writes.
inline cudaError_t launch_dependent(const void* fn, unsigned grid, unsigned threads,
	size_t smem, cudaStream_t stream, void** args)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(threads);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace grav
