// probe.cu -- measured FP32 FMA throughput of the active GPU, used as the
// denominator of the all-pairs kernels' roofline (they are FP32-pipe bound;
// the device's HBM and tensor peaks do not bound them).
//
// Every thread runs 8 independent FMA chains; the grid fills every SM with
// 8 CTAs of 256 threads. Flops counted: 2 per FMA.
#include <algorithm>
#include <string>

#include "cvortex/cvtx_gb300.h"
#include "nbody.h"
#include "runtime.h"

namespace cvtx {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, float a, float b) {
	float x[kChains];
#pragma unroll
	for (int c = 0; c < kChains; ++c) x[c] = float(threadIdx.x + c);
#pragma unroll 4
	for (int i = 0; i < kIters; ++i) {
#pragma unroll
		for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
	}
	float s = 0.f;
#pragma unroll
	for (int c = 0; c < kChains; ++c) s += x[c];
	if (s == 1.2345f) out[threadIdx.x] = s;   // keeps the chains live
}

// The same with packed two-wide FP32 FMAs (fma.rn.f32x2): one instruction
// performs two FMAs, so the FMA peak is reached with half the issue slots.
__global__ void __launch_bounds__(256) fma2_probe_kernel(float* out, float a, float b) {
	float2 x[kChains / 2];
	const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
#pragma unroll
	for (int c = 0; c < kChains / 2; ++c) x[c] = make_float2(float(threadIdx.x + c), float(c));
#pragma unroll 4
	for (int i = 0; i < kIters; ++i) {
#pragma unroll
		for (int c = 0; c < kChains / 2; ++c) x[c] = __ffma2_rn(x[c], a2, b2);
	}
	float s = 0.f;
#pragma unroll
	for (int c = 0; c < kChains / 2; ++c) s += x[c].x + x[c].y;
	if (s == 1.2345f) out[threadIdx.x] = s;
}

// Mixed issue: P packed (f32x2) and S scalar FMA chains per thread. Tells
// whether scalar FMAs can run beside packed ones (on a separate FMA pipe),
// which bounds what a kernel mixing both can reach.
template <int P, int S>
__global__ void __launch_bounds__(256) fma_mix_probe_kernel(float* out, float a, float b) {
	float2 x[P > 0 ? P : 1];
	float y[S > 0 ? S : 1];
	const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
#pragma unroll
	for (int c = 0; c < P; ++c) x[c] = make_float2(float(threadIdx.x + c), float(c));
#pragma unroll
	for (int c = 0; c < S; ++c) y[c] = float(threadIdx.x + 3 * c);
#pragma unroll 4
	for (int i = 0; i < kIters; ++i) {
#pragma unroll
		for (int c = 0; c < P; ++c) x[c] = __ffma2_rn(x[c], a2, b2);
#pragma unroll
		for (int c = 0; c < S; ++c) y[c] = fmaf(y[c], a, b);
	}
	float s = 0.f;
#pragma unroll
	for (int c = 0; c < P; ++c) s += x[c].x + x[c].y;
#pragma unroll
	for (int c = 0; c < S; ++c) s += y[c];
	if (s == 1.2345f) out[threadIdx.x] = s;
}

double run_probe(DeviceContext* c, float* out, cudaEvent_t e0, cudaEvent_t e1, int repeats,
	bool packed, cudaError_t& e) {
	const int blocks = c->num_sms * 8;
	double best = 0.0;
	for (int r = 0; r <= repeats && e == cudaSuccess; ++r) {
		cudaEventRecord(e0, c->stream);
		if (packed) fma2_probe_kernel<<<blocks, 256, 0, c->stream>>>(out, 0.999f, 1e-3f);
		else fma_probe_kernel<<<blocks, 256, 0, c->stream>>>(out, 0.999f, 1e-3f);
		count_launch();
		cudaEventRecord(e1, c->stream);
		e = cudaEventSynchronize(e1);
		float ms = 0.f;
		if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
		const double flops = 2.0 * kChains * double(kIters) * 256.0 * blocks;
		if (r > 0 && ms > 0.f) best = std::max(best, flops / (double(ms) * 1e-3) / 1e12);
	}
	return best;
}

}  // namespace
}  // namespace cvtx

// Both probes, best of `repeats` timed launches each (2 flops per FMA).
extern "C" CVTX_EXPORT int cvtx_gb300_probe_fp32_detail(int repeats, double* scalar_fma,
	double* packed_fma) {
	using namespace cvtx;
	if (!scalar_fma || !packed_fma || repeats < 1) return -1;
	std::lock_guard<std::recursive_mutex> g(Runtime::get().lock());
	DeviceContext* c = Runtime::get().active_context();
	if (!c) return -3;
	float* out = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	cudaError_t e = cudaMalloc(&out, 256 * sizeof(float));
	if (e == cudaSuccess) e = cudaEventCreate(&e0);
	if (e == cudaSuccess) e = cudaEventCreate(&e1);
	double scalar = 0.0, packed = 0.0;
	if (e == cudaSuccess) scalar = run_probe(c, out, e0, e1, repeats, false, e);
	if (e == cudaSuccess) packed = run_probe(c, out, e0, e1, repeats, true, e);
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	if (out) cudaFree(out);
	if (e != cudaSuccess) {
		set_error(std::string("cvtx_gb300_probe_fp32: ") + cudaGetErrorString(e));
		return -2;
	}
	*scalar_fma = scalar;
	*packed_fma = packed;
	return 0;
}

// Mixed packed / scalar FMA probe: `packed` f32x2 chains and `scalar` chains
// per thread, (packed, scalar) in {(4,0), (0,8), (2,4), (3,2), (2,2), (4,4),
// (1,6), (4,2), (6,3)}. Best of `repeats` launches, TFLOP/s (2 flops per FMA).
extern "C" CVTX_EXPORT int cvtx_gb300_probe_fp32_mix(int packed, int scalar, int repeats,
	double* tflops) {
	using namespace cvtx;
	if (!tflops || repeats < 1) return -1;
	using K = void (*)(float*, float, float);
	K k = nullptr;
	if (packed == 4 && scalar == 0) k = fma_mix_probe_kernel<4, 0>;
	else if (packed == 0 && scalar == 8) k = fma_mix_probe_kernel<0, 8>;
	else if (packed == 2 && scalar == 4) k = fma_mix_probe_kernel<2, 4>;
	else if (packed == 3 && scalar == 2) k = fma_mix_probe_kernel<3, 2>;
	else if (packed == 2 && scalar == 2) k = fma_mix_probe_kernel<2, 2>;
	else if (packed == 4 && scalar == 4) k = fma_mix_probe_kernel<4, 4>;
	else if (packed == 1 && scalar == 6) k = fma_mix_probe_kernel<1, 6>;
	else if (packed == 4 && scalar == 2) k = fma_mix_probe_kernel<4, 2>;
	else if (packed == 6 && scalar == 3) k = fma_mix_probe_kernel<6, 3>;
	if (!k) return -1;
	std::lock_guard<std::recursive_mutex> g(Runtime::get().lock());
	DeviceContext* c = Runtime::get().active_context();
	if (!c) return -3;
	float* out = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	cudaError_t e = cudaMalloc(&out, 256 * sizeof(float));
	if (e == cudaSuccess) e = cudaEventCreate(&e0);
	if (e == cudaSuccess) e = cudaEventCreate(&e1);
	const int blocks = c->num_sms * 8;
	double best = 0.0;
	for (int r = 0; r <= repeats && e == cudaSuccess; ++r) {
		cudaEventRecord(e0, c->stream);
		k<<<blocks, 256, 0, c->stream>>>(out, 0.999f, 1e-3f);
		count_launch();
		cudaEventRecord(e1, c->stream);
		e = cudaEventSynchronize(e1);
		float ms = 0.f;
		if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
		const double flops = 2.0 * (2 * packed + scalar) * double(kIters) * 256.0 * blocks;
		if (r > 0 && ms > 0.f) best = std::max(best, flops / (double(ms) * 1e-3) / 1e12);
	}
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	if (out) cudaFree(out);
	if (e != cudaSuccess) {
		set_error(std::string("cvtx_gb300_probe_fp32_mix: ") + cudaGetErrorString(e));
		return -2;
	}
	*tflops = best;
	return 0;
}

// The FP32 FMA peak: the larger of the two probes.
extern "C" CVTX_EXPORT int cvtx_gb300_probe_fp32_tflops(int repeats, double* tflops) {
	if (!tflops) return -1;
	double a = 0.0, b = 0.0;
	const int rc = cvtx_gb300_probe_fp32_detail(repeats, &a, &b);
	if (rc == 0) *tflops = a > b ? a : b;
	return rc;
}
