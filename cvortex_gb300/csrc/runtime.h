// runtime.h -- single-process CUDA device state behind the cvtx_ ABI.
//
// Replaces the reference's OpenCL runtime (src/opencl_acc.cpp,
// src/OclPlatformState.cpp, src/OclDeviceState.cpp): enumerates CUDA devices,
// keeps the list of enabled accelerators (accelerator ids = CUDA ordinals),
// and owns, per device, one non-blocking stream plus grow-only device and
// pinned host buffers reused across calls. All GPU work runs on the first
// enabled accelerator, as in the reference (src/ocl_P3D.cpp:46).
#pragma once
#include <cstddef>
#include <mutex>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "nbody.h"

namespace cvtx {

// Makes `dev` current for a scope and restores the caller's current device
// afterwards, so that entry points working on an object's own device leave
// the calling thread's device as they found it.
struct DeviceGuard {
	int prev = -1;
	explicit DeviceGuard(int dev) {
		if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
		if (dev >= 0 && dev != prev) cudaSetDevice(dev);
	}
	~DeviceGuard() {
		int cur = -1;
		if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
	}
	DeviceGuard(const DeviceGuard&) = delete;
	DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// Grow-only device allocation (256-byte aligned by cudaMalloc).
struct DevBuf {
	void* ptr = nullptr;
	size_t bytes = 0;
	cudaError_t ensure(size_t need);
	void release();
};

// Grow-only pinned host allocation.
struct HostBuf {
	void* ptr = nullptr;
	size_t bytes = 0;
	cudaError_t ensure(size_t need);
	void release();
};

struct DeviceContext {
	int device = -1;
	int num_sms = 0;
	cudaStream_t stream = nullptr;
	unsigned* d_err = nullptr;      // device error word of the host-pointer calls
	unsigned* h_err = nullptr;      // pinned copy
	unsigned* d_err_dev = nullptr;  // device error word of the device-pointer calls
	// Orders every user of `ws` (host-pointer calls on `stream`, device-pointer
	// calls on their callers' streams): each waits on it before its first
	// launch and records it after its last.
	cudaEvent_t ws_ev = nullptr;
	DevBuf src, tgt, out0, out1, ws;
	DevBuf redist;                  // particle redistribution scratch (grow-only)
	HostBuf h_redist;               // its cells, pinned (grow-only)
	HostBuf h_src, h_tgt, h_out0, h_out1;
	cudaError_t open(int dev);
	void close();
	LaunchEnv env() const;
	// Make sure the workspace holds `bytes`.
	cudaError_t ensure_ws(size_t bytes) { return ws.ensure(bytes); }
	// The workspace for `want` bytes or, if that cannot be allocated, for
	// `fallback` bytes (the launchers then take a form that fits it).
	cudaError_t ensure_ws_or(size_t want, size_t fallback) {
		const cudaError_t e = ws.ensure(want);
		if (e == cudaSuccess || fallback >= want) return e;
		(void)cudaGetLastError();   // the failed allocation is not the call's error
		return ws.ensure(fallback);
	}
};

class Runtime {
 public:
	static Runtime& get();

	void initialise();
	void finalise();
	bool is_initialised();
	int num_devices();
	const char* device_name(int id);
	int num_enabled();
	bool enabled(int id);
	void enable(int id);
	void disable(int id);
	const char* information();

	// Context of the first enabled accelerator (opened on first use) or
	// nullptr when none is enabled. The caller must hold lock().
	DeviceContext* active_context();
	std::recursive_mutex& lock() { return mu_; }

 private:
	Runtime() = default;
	void enumerate_locked();
	std::recursive_mutex mu_;
	bool initialised_ = false;
	bool enumerated_ = false;
	std::vector<std::string> names_;
	std::vector<int> active_;
	std::vector<DeviceContext*> ctx_;
	std::string info_;
};

// Error reporting for the GPU path (the reference ABI functions return void).
// Text of a nonzero device error word (the kErr* bits of common.cuh).
std::string device_error_text(unsigned word);
void set_error(const std::string& msg);
void clear_error();
const char* last_error();

}  // namespace cvtx
