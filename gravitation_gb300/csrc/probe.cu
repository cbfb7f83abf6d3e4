// probe.cu -- FP32 FMA-pipe throughput probe (roofline denominator for stage 1).
//
// Each thread runs 8 independent FFMA chains; with 256 threads per CTA and enough
// CTAs to fill every SM, the kernel issues one FFMA per clock per SM sub-partition,
// i.e. it measures the FP32 FMA rate (SMs x 128 x 2 FLOP per clock) at the clock the
// GPU actually runs.  The caller times it with CUDA events; one launch performs
// blocks * 256 * iters * 8 * 16 FMAs.
#include "grav_types.h"

namespace grav {

__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, int iters)
{
	float a[8];
	const float b = 0.999999f, c = 1e-7f;
#pragma unroll
	for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 1e-3f + i;
	for (int it = 0; it < iters; ++it) {
#pragma unroll
		for (int u = 0; u < 16; ++u) {
#pragma unroll
			for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], b, c);
		}
	}
	float s = 0.f;
#pragma unroll
	for (int i = 0; i < 8; ++i) s += a[i];
	out[static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

}  // namespace grav

extern "C" int grav_fp32_peak_probe(float* out, int32_t blocks, int32_t iters, void* stream)
{
	if (!out || blocks <= 0 || iters <= 0) return GRAV_E_ARG;
	grav::fma_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(out, iters);
	return cudaGetLastError() == cudaSuccess ? GRAV_OK : GRAV_E_CUDA;
}
