// grav_types.h -- internal constants shared by host and device code of libgravgb300.
#pragma once

#include "gravitation_gb300.h"

// Wall-clock bound of every device-side wait on a bulk copy (nanoseconds).
#define GRAV_WAIT_NS 2000000000ull

namespace grav {

// Launch-time view of one stage-1 kernel instantiation.
struct Stage1Kernel {
	int mode, bpt, threads, jtile;
	const void* fn;       // __global__ function
	int smem_bytes;       // dynamic shared memory per CTA
};

// Kernel tables, one per translation unit (stage1_f32.cu, stage1_f64.cu).
int stage1_table_f32(const Stage1Kernel** out);
int stage1_table_f64(const Stage1Kernel** out);
int stage1_table_sym(const Stage1Kernel** out);

}  // namespace grav
