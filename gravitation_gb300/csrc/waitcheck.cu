// waitcheck.cu -- test hook for the bounded-wait failure path of the stage-1 kernels.
//
// Every device-side wait of the library (an mbarrier phase completed by a bulk copy) is
// bounded in time; when the bound expires the CTA records GRAV_DEV_TIMEOUT in the
// caller's error flag and returns, so a lost copy never hangs the GPU and the context
// stays usable.  This kernel exercises exactly that path without any fault: one CTA
// initialises an mbarrier that nothing ever arrives on (no copy is issued), waits on it
// with the same bounded wait and a caller-chosen limit, agrees on the outcome with
// __syncthreads_or like the stage-1 kernels, records the error and returns.
#include "grav_device.cuh"

namespace grav {

__global__ void __launch_bounds__(128) wait_timeout_kernel(int32_t* err, uint64_t limit_ns)
{
	__shared__ __align__(8) uint64_t bar;
	if (threadIdx.x == 0) {
		mbar_init(&bar, 1);
		fence_barrier_init();
	}
	__syncthreads();
	const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
	if (__syncthreads_or(!ok)) {
		if (threadIdx.x == 0) set_error(err, GRAV_DEV_TIMEOUT);
		return;
	}
}

int record_error(int code, const char* msg);

}  // namespace grav

extern "C" int grav_wait_check(int32_t* err, int64_t limit_ns, void* stream)
{
	if (!err) return grav::record_error(GRAV_E_ARG, "NULL err");
	if (limit_ns <= 0 || limit_ns > static_cast<int64_t>(GRAV_WAIT_NS))
		return grav::record_error(GRAV_E_ARG, "limit_ns must be in (0, 2e9]");
	grav::wait_timeout_kernel<<<1, 128, 0, static_cast<cudaStream_t>(stream)>>>(
		err, static_cast<uint64_t>(limit_ns));
	cudaError_t e = cudaGetLastError();
	return e == cudaSuccess ? GRAV_OK : grav::record_error(GRAV_E_CUDA, cudaGetErrorString(e));
}
