// selftest.cu -- on-device check of the bounded-wait error path.
//
// Every mbarrier wait of the all-pairs kernels is bounded: on expiry the
// kernel sets the error word, drains its copies and returns, and the host
// reports the error (the reference instead falls back to the CPU silently,
// src/P3D.cpp:356-363). This kernel exercises that path without a fault: one
// CTA waits on an mbarrier that nothing will ever complete (a withheld
// doorbell) with a short limit, records the expiry in the error word, and
// returns; no copy is in flight, so the context stays usable.
#include <string>

#include "common.cuh"
#include "cvortex/cvtx_gb300.h"
#include "nbody.h"
#include "runtime.h"

namespace cvtx {
namespace {

__global__ void withheld_doorbell_kernel(unsigned* err, unsigned long long limit_ns) {
	__shared__ __align__(8) uint64_t bar;
	if (threadIdx.x == 0) {
		mbar_init(&bar, 1u);    // expects one arrival that never comes
		mbar_init_fence();
	}
	__syncthreads();
	const bool ok = mbar_wait_for(&bar, 0u, limit_ns);
	if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(err, kErrPipelineTimeout);
}

}  // namespace
}  // namespace cvtx

using namespace cvtx;

extern "C" {

CVTX_EXPORT int cvtx_gb300_selftest_withheld_wait(double limit_ms) {
	if (!(limit_ms > 0.0 && limit_ms <= 1000.0)) return -1;
	std::lock_guard<std::recursive_mutex> g(Runtime::get().lock());
	DeviceContext* c = Runtime::get().active_context();
	if (!c) return -3;
	unsigned* d = nullptr;
	unsigned w = 0;
	cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d), sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(unsigned), c->stream);
	if (e == cudaSuccess) {
		withheld_doorbell_kernel<<<1, 64, 0, c->stream>>>(
			d, static_cast<unsigned long long>(limit_ms * 1e6));
		count_launch();
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(&w, d, sizeof w, cudaMemcpyDeviceToHost, c->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
	if (d) cudaFree(d);
	if (e != cudaSuccess) {
		set_error(std::string("cvtx_gb300_selftest_withheld_wait: ") + cudaGetErrorString(e));
		return -2;
	}
	return static_cast<int>(w);
}

}  // extern "C"
