// runtime.cpp -- CUDA device state, accelerator API and error query.
//
// Accelerator API semantics follow the reference (src/accelerators.cpp:39-118,
// src/opencl_acc.cpp:55-258):
//  * cvtx_initialise() enumerates the GPUs once and (on every call) adds the
//    default accelerator 0 to the enabled list if it is not there;
//  * cvtx_finalise() releases device resources and clears the enabled list;
//  * accelerator ids index the GPUs; enabling twice is a no-op;
//  * with no enabled accelerator the M2M functions run on the host.
#include "runtime.h"

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "cvortex/libcvtx.h"
#include "cvortex/cvtx_gb300.h"

namespace cvtx {

// ---- buffers ---------------------------------------------------------------
// CVTX_GB300_WS_LIMIT (bytes): device buffers larger than this fail as an
// out-of-memory cudaMalloc would (host-side fault injection for the tests of
// the workspace fallbacks; unset, no limit).
static size_t devbuf_limit() {
	static const size_t lim = [] {
		const char* e = std::getenv("CVTX_GB300_WS_LIMIT");
		const long long v = (e && *e) ? std::atoll(e) : 0;
		return v > 0 ? size_t(v) : SIZE_MAX;
	}();
	return lim;
}

cudaError_t DevBuf::ensure(size_t need) {
	if (need <= bytes && ptr) return cudaSuccess;
	if (need > devbuf_limit()) return cudaErrorMemoryAllocation;
	if (need == 0) need = 256;
	release();
	size_t grow = need + need / 4;
	cudaError_t e = grow <= devbuf_limit() ? cudaMalloc(&ptr, grow) : cudaErrorMemoryAllocation;
	if (e != cudaSuccess) {
		(void)cudaGetLastError();   // retried at the size needed
		ptr = nullptr;
		bytes = 0;
		e = cudaMalloc(&ptr, need);
		if (e != cudaSuccess) { ptr = nullptr; return e; }
		grow = need;
	}
	bytes = grow;
	return cudaSuccess;
}
void DevBuf::release() {
	if (ptr) cudaFree(ptr);
	ptr = nullptr;
	bytes = 0;
}
cudaError_t HostBuf::ensure(size_t need) {
	if (need <= bytes && ptr) return cudaSuccess;
	if (need == 0) need = 256;
	release();
	size_t grow = need + need / 4;
	cudaError_t e = cudaMallocHost(&ptr, grow);
	if (e != cudaSuccess) { ptr = nullptr; return e; }
	bytes = grow;
	return cudaSuccess;
}
void HostBuf::release() {
	if (ptr) cudaFreeHost(ptr);
	ptr = nullptr;
	bytes = 0;
}

cudaError_t DeviceContext::open(int dev) {
	device = dev;
	cudaError_t e = cudaSetDevice(dev);
	if (e != cudaSuccess) return e;
	e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
	if (e != cudaSuccess) return e;
	e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
	if (e != cudaSuccess) return e;
	e = cudaMalloc(reinterpret_cast<void**>(&d_err), sizeof(unsigned));
	if (e != cudaSuccess) return e;
	e = cudaMalloc(reinterpret_cast<void**>(&d_err_dev), sizeof(unsigned));
	if (e != cudaSuccess) return e;
	e = cudaMallocHost(reinterpret_cast<void**>(&h_err), sizeof(unsigned));
	if (e != cudaSuccess) return e;
	*h_err = 0u;
	e = cudaEventCreateWithFlags(&ws_ev, cudaEventDisableTiming);
	if (e != cudaSuccess) return e;
	e = cudaMemset(d_err_dev, 0, sizeof(unsigned));
	if (e != cudaSuccess) return e;
	return cudaMemset(d_err, 0, sizeof(unsigned));
}

void DeviceContext::close() {
	if (device >= 0) cudaSetDevice(device);
	if (stream) cudaStreamSynchronize(stream);
	src.release(); tgt.release(); out0.release(); out1.release(); ws.release();
	redist.release();
	h_redist.release();
	h_src.release(); h_tgt.release(); h_out0.release(); h_out1.release();
	if (d_err) cudaFree(d_err);
	if (d_err_dev) cudaFree(d_err_dev);
	if (h_err) cudaFreeHost(h_err);
	if (ws_ev) cudaEventDestroy(ws_ev);
	if (stream) cudaStreamDestroy(stream);
	d_err = nullptr; d_err_dev = nullptr; h_err = nullptr; ws_ev = nullptr; stream = nullptr;
}

LaunchEnv DeviceContext::env() const {
	LaunchEnv e;
	e.ws = ws.ptr;
	e.ws_bytes = ws.bytes;
	e.err = d_err;
	e.stream = stream;
	e.num_sms = num_sms;
	return e;
}

// ---- runtime -----------------------------------------------------------------
Runtime& Runtime::get() {
	static Runtime* rt = new Runtime();   // never destroyed: safe at exit
	return *rt;
}

void Runtime::enumerate_locked() {
	if (enumerated_) return;
	enumerated_ = true;
	names_.clear();
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) {
		n = 0;
		cudaGetLastError();   // clear the sticky "no device" status
	}
	for (int i = 0; i < n; ++i) {
		cudaDeviceProp prop;
		if (cudaGetDeviceProperties(&prop, i) == cudaSuccess) names_.emplace_back(prop.name);
		else names_.emplace_back("CUDA device");
	}
	ctx_.assign(names_.size(), nullptr);
}

static std::string compiler_string() {
#if defined(__clang__)
	return "clang " + std::to_string(__clang_major__) + "." + std::to_string(__clang_minor__);
#elif defined(__GNUC__)
	return "GCC " + std::to_string(__GNUC__) + "." + std::to_string(__GNUC_MINOR__) + "." +
		std::to_string(__GNUC_PATCHLEVEL__);
#else
	return "Unknown compiler";
#endif
}

void Runtime::initialise() {
	std::lock_guard<std::recursive_mutex> g(mu_);
	enumerate_locked();
	initialised_ = true;
	if (!names_.empty() && std::find(active_.begin(), active_.end(), 0) == active_.end())
		active_.push_back(0);
	int rt_ver = 0;
	cudaRuntimeGetVersion(&rt_ver);
	info_ = "cvortex version: 0.3.8 (GB300 CUDA build)\n";
	info_ += "compiler: " + compiler_string() + "\n";
#ifdef _OPENMP
	info_ += "using OpenMP: TRUE\n";
#else
	info_ += "using OpenMP: FALSE\n";
#endif
	info_ += "using OpenCL: FALSE\n";
	info_ += "using CUDA: TRUE (runtime " + std::to_string(rt_ver / 1000) + "." +
		std::to_string((rt_ver % 1000) / 10) + ", kernels for sm_103a)\n";
	for (size_t i = 0; i < names_.size(); ++i)
		info_ += "accelerator " + std::to_string(i) + ": " + names_[i] + "\n";
}

void Runtime::finalise() {
	std::lock_guard<std::recursive_mutex> g(mu_);
	for (auto*& c : ctx_) {
		if (c) { c->close(); delete c; c = nullptr; }
	}
	active_.clear();
	initialised_ = false;
	info_.clear();
}

bool Runtime::is_initialised() {
	std::lock_guard<std::recursive_mutex> g(mu_);
	return initialised_;
}

int Runtime::num_devices() {
	std::lock_guard<std::recursive_mutex> g(mu_);
	enumerate_locked();
	return int(names_.size());
}

const char* Runtime::device_name(int id) {
	std::lock_guard<std::recursive_mutex> g(mu_);
	enumerate_locked();
	if (id < 0 || id >= int(names_.size())) return nullptr;
	return names_[id].c_str();
}

int Runtime::num_enabled() {
	std::lock_guard<std::recursive_mutex> g(mu_);
	return int(active_.size());
}

bool Runtime::enabled(int id) {
	std::lock_guard<std::recursive_mutex> g(mu_);
	return std::find(active_.begin(), active_.end(), id) != active_.end();
}

void Runtime::enable(int id) {
	std::lock_guard<std::recursive_mutex> g(mu_);
	enumerate_locked();
	if (id < 0 || id >= int(names_.size())) return;
	if (std::find(active_.begin(), active_.end(), id) == active_.end()) active_.push_back(id);
}

void Runtime::disable(int id) {
	std::lock_guard<std::recursive_mutex> g(mu_);
	auto it = std::find(active_.begin(), active_.end(), id);
	if (it != active_.end()) active_.erase(it);
}

const char* Runtime::information() {
	std::lock_guard<std::recursive_mutex> g(mu_);
	return info_.c_str();
}

DeviceContext* Runtime::active_context() {
	if (active_.empty()) return nullptr;
	const int dev = active_.front();
	if (dev < 0 || dev >= int(ctx_.size())) return nullptr;
	if (!ctx_[dev]) {
		auto* c = new DeviceContext();
		const cudaError_t e = c->open(dev);
		if (e != cudaSuccess) {
			set_error(std::string("opening CUDA device failed: ") + cudaGetErrorString(e));
			c->close();
			delete c;
			return nullptr;
		}
		ctx_[dev] = c;
	}
	cudaSetDevice(dev);
	return ctx_[dev];
}

// ---- error reporting -------------------------------------------------------
std::string device_error_text(unsigned w) {
	std::string t;
	auto add = [&](unsigned bit, const char* what) {
		if (!(w & bit)) return;
		if (!t.empty()) t += ", ";
		t += what;
	};
	add(1u, "a device-side wait expired");
	add(2u, "draining copies after an expired wait timed out");
	add(4u, "a misaligned bulk copy was skipped");
	add(8u, "launch shape or shared-memory alignment not as expected");
	add(16u, "a work item was out of range");
	if (t.empty()) t = "device error";
	return t + " (code " + std::to_string(w) + ")";
}

static std::mutex g_err_mu;
static std::string g_err;

void set_error(const std::string& msg) {
	std::lock_guard<std::mutex> g(g_err_mu);
	if (g_err.empty()) std::fprintf(stderr, "cvortex (GB300): %s\n", msg.c_str());
	g_err = msg;
}
void clear_error() {
	std::lock_guard<std::mutex> g(g_err_mu);
	g_err.clear();
}
const char* last_error() {
	static thread_local std::string copy;
	std::lock_guard<std::mutex> g(g_err_mu);
	copy = g_err;
	return copy.c_str();
}

// ---- shared knobs ------------------------------------------------------------
static std::atomic<unsigned long long> g_launches{0};
void count_launch(int n) { g_launches.fetch_add(static_cast<unsigned long long>(n)); }
unsigned long long launch_count() { return g_launches.load(); }

static std::atomic<float> g_rho_c{0.5f};
float gaussian_rho_c() { return g_rho_c.load(); }
void set_gaussian_rho_c(float r) { g_rho_c.store(r); }

int reg_from_tag(const char* tag) {
	if (!tag) return -1;
	char t[33];
	std::memcpy(t, tag, 32);
	t[32] = '\0';
	if (!std::strcmp(t, "singular")) return 0;
	if (!std::strcmp(t, "winckelmans")) return 1;
	if (!std::strcmp(t, "planetary")) return 2;
	if (!std::strcmp(t, "gaussian")) return 3;
	return -1;
}

}  // namespace cvtx

// ---- C ABI: accelerator control (reference libcvtx.h:101-110) -----------------
using cvtx::Runtime;

extern "C" {

CVTX_EXPORT void cvtx_initialise() { Runtime::get().initialise(); }
CVTX_EXPORT void cvtx_finalise() { Runtime::get().finalise(); }
CVTX_EXPORT const char* cvtx_information() { return Runtime::get().information(); }
CVTX_EXPORT int cvtx_num_accelerators() { return Runtime::get().num_devices(); }
CVTX_EXPORT int cvtx_num_enabled_accelerators() { return Runtime::get().num_enabled(); }
CVTX_EXPORT const char* cvtx_accelerator_name(int id) { return Runtime::get().device_name(id); }
CVTX_EXPORT int cvtx_accelerator_enabled(int id) { return Runtime::get().enabled(id) ? 1 : 0; }
CVTX_EXPORT void cvtx_accelerator_enable(int id) { Runtime::get().enable(id); }
CVTX_EXPORT void cvtx_accelerator_disable(int id) { Runtime::get().disable(id); }

CVTX_EXPORT const char* cvtx_gb300_last_error(void) { return cvtx::last_error(); }
CVTX_EXPORT void cvtx_gb300_clear_error(void) { cvtx::clear_error(); }
CVTX_EXPORT unsigned long long cvtx_gb300_kernel_launches(void) { return cvtx::launch_count(); }
CVTX_EXPORT float cvtx_gb300_gaussian_rho_c(void) { return cvtx::gaussian_rho_c(); }
CVTX_EXPORT void cvtx_gb300_set_gaussian_rho_c(float rho_c) {
	if (rho_c >= 0.f && rho_c <= 1.f) cvtx::set_gaussian_rho_c(rho_c);
}

}  // extern "C"
