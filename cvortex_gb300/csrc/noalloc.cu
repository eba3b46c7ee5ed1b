// noalloc.cu -- P3D velocity / vortex stretching on device records without
// any device allocation: cvtx_gb300_dev_P3D_M2M_noalloc.
//
// Who needs it: callers that cannot let a library call cudaMalloc. Examples
// are a solver whose device memory is carved out of one pool reserved at
// start-up (an allocation inside the call would bypass its accounting and can
// fail once the pool holds the whole GPU), and a time-stepping loop that
// cannot absorb the latency and device-wide synchronisation that
// cudaMalloc / cudaFree bring. This entry point touches only the caller's
// buffers and a fixed scratch area that is part of the library image.
//
// Scratch: g_scratch below, 32 MiB in every GPU's memory for as long as the
// library stays loaded. It holds the FP64 partial sums of source splits. The
// split count is capped so the partials fit, which admits up to
// kMaxTargets = 233,016 targets (two splits of the fused kernel's nine
// partials). Larger target counts are rejected with an error; the number of
// sources is not limited.
//
// Sharing: every call on a device uses the same scratch and error word and
// leaves its contents behind. Each split partial is written before the
// finalize kernel reads it, so no stale partial is ever used; the error word
// is cleared at the start of each call. Calls whose work overlaps on the GPU
// (different streams, or host threads that do not order their streams) race
// on the scratch and must not be issued.
//
// Set-up: the first call on a device, with that device current, resolves the
// device addresses of the scratch and the error word (cudaGetSymbolAddress)
// and reads the SM count; later calls reuse them. Make that first call before
// any stream capture is started on the device.
#include <cstdio>
#include <mutex>
#include <string>

#include "cvortex/cvtx_gb300.h"
#include "nbody.h"
#include "runtime.h"

namespace cvtx {
namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;
constexpr int kMaxTargets = int(kScratchBytes / (2 * 9 * sizeof(double)));   // 233,016
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];
static __device__ __align__(256) unsigned g_err_word;

struct DeviceSlot {
	bool ready = false;
	void* scratch = nullptr;
	unsigned* err = nullptr;
	int num_sms = 0;
};

std::mutex g_mu;
DeviceSlot g_slots[kMaxDevices];

// After a device-side wait expired (g_err_word != 0) the kernels return
// without writing; make that visible in the outputs.
__global__ void poison_on_error(float* vel, float* dvort, int n) {
	if (g_err_word == 0u) return;
	const float nan = __int_as_float(0x7fc00000);
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += gridDim.x * blockDim.x) {
		if (vel) vel[i] = nan;
		if (dvort) dvort[i] = nan;
	}
}

int fail(const std::string& msg, int code) {
	set_error("cvtx_gb300_dev_P3D_M2M_noalloc: " + msg);
	return code;
}

}  // namespace
}  // namespace cvtx

using namespace cvtx;

extern "C" CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_noalloc(const void* src, int n_src,
	const void* tgt, int tgt_stride, int n_tgt, float* vel_out, float* dvort_out, int reg,
	float regularisation_radius, void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_src < 0 || !tgt || (n_src > 0 && !src) || reg < 0 || reg > 3 ||
		(!vel_out && !dvort_out) || tgt_stride < 1 || (dvort_out && tgt_stride < 2))
		return fail("invalid argument", -1);
	if (n_tgt > kMaxTargets)
		return fail(std::to_string(n_tgt) + " targets exceed the " +
			std::to_string(kMaxTargets) + "-target limit of its fixed 32 MiB scratch", -1);

	int dev = -1;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return fail(cudaGetErrorString(e), -2);
	if (dev < 0 || dev >= kMaxDevices) return fail("device ordinal out of range", -1);
	DeviceSlot slot;
	{
		std::lock_guard<std::mutex> g(g_mu);
		DeviceSlot& s = g_slots[dev];
		if (!s.ready) {
			e = cudaGetSymbolAddress(&s.scratch, g_scratch);
			if (e == cudaSuccess)
				e = cudaGetSymbolAddress(reinterpret_cast<void**>(&s.err), g_err_word);
			if (e == cudaSuccess)
				e = cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev);
			if (e != cudaSuccess) return fail(std::string("set-up: ") + cudaGetErrorString(e), -2);
			s.ready = true;
		}
		slot = s;
	}
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	e = cudaMemsetAsync(slot.err, 0, sizeof(unsigned), st);
	if (e != cudaSuccess) return fail(cudaGetErrorString(e), -2);

	LaunchEnv env;
	env.ws = slot.scratch;
	env.ws_bytes = kScratchBytes;
	env.err = slot.err;
	env.stream = st;
	env.num_sms = slot.num_sms;
	P3DInduceProblem p;
	p.src = static_cast<const float4*>(src); p.n_src = n_src;
	p.tgt = static_cast<const float4*>(tgt); p.tstride = tgt_stride; p.n_tgt = n_tgt;
	p.out_vel = vel_out; p.out_dvort = dvort_out; p.sigma = regularisation_radius;
	const unsigned ops = (vel_out ? kOpVel : 0u) | (dvort_out ? kOpDvort : 0u);
	e = p3d_induce_bounded(reg, ops, p, env);
	if (e != cudaSuccess) return fail(cudaGetErrorString(e), -2);
	const int blocks = (3 * n_tgt + 255) / 256 < slot.num_sms * 4 ? (3 * n_tgt + 255) / 256
	                                                               : slot.num_sms * 4;
	poison_on_error<<<blocks, 256, 0, st>>>(vel_out, dvort_out, n_tgt);
	count_launch();
	e = cudaGetLastError();
	return e == cudaSuccess ? 0 : fail(cudaGetErrorString(e), -2);
}
