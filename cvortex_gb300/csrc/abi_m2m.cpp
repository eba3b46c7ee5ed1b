// abi_m2m.cpp -- the M2M entry points of the cvtx_ ABI and the GB300
// extensions that take host pointers.
//
// Dispatch (reference gates: src/P3D.cpp:352-364, src/P2D.cpp:150-161,
// src/F3D.cpp:169-201):
//   * an accelerator is enabled and the regularisation tag names a GPU kernel
//     -> CUDA path on the first enabled accelerator, for every problem size
//        (the reference's 256-particle and "CPU is better" gates existed to
//        amortise its per-chunk OpenCL launches and are not needed here);
//   * no accelerator enabled, or a tag with no GPU kernel -> host loops.
// The CUDA path never falls back to the host: on any CUDA error or device
// timeout it records the message (cvtx_gb300_last_error), prints it once to
// stderr and fills the caller's result array with NaN.
//
// CUDA path of one call: gather the pointer array into pinned float4 records
// (OpenMP over records for large sets), one H2D copy per array, the kernel(s)
// on the context's stream, one D2H copy of the packed result plus the device
// error word, then a copy into the caller's array.
#include <cmath>
#include <cstring>
#include <limits>
#include <string>

#include "cvortex/libcvtx.h"
#include "cvortex/cvtx_gb300.h"
#include "host_paths.h"
#include "nbody.h"
#include "runtime.h"

namespace cvtx {
namespace {

constexpr int kParallelGather = 32768;
// Velocity calls with at least this many points compare the points with the
// sources' coordinates, to use the source records as the targets.
constexpr int kSelfCheckMin = 16384;

void gather_p3d_host(const cvtx_P3D* const* src, int n, float4* out) {
#pragma omp parallel for schedule(static) if (n >= kParallelGather)
	for (int i = 0; i < n; ++i) {
		const cvtx_P3D* p = src[i];
		out[2 * i] = make_float4(p->coord.x[0], p->coord.x[1], p->coord.x[2], p->volume);
		out[2 * i + 1] = make_float4(p->vorticity.x[0], p->vorticity.x[1], p->vorticity.x[2], 0.f);
	}
}
void pack_v3_host(const bsv_V3f* v, int n, float4* out) {
#pragma omp parallel for schedule(static) if (n >= kParallelGather)
	for (int i = 0; i < n; ++i) out[i] = make_float4(v[i].x[0], v[i].x[1], v[i].x[2], 0.f);
}
void gather_p2d_host(const cvtx_P2D* const* src, int n, float4* out) {
#pragma omp parallel for schedule(static) if (n >= kParallelGather)
	for (int i = 0; i < n; ++i) {
		const cvtx_P2D* p = src[i];
		out[i] = make_float4(p->coord.x[0], p->coord.x[1], p->vorticity, p->area);
	}
}
void pack_v2_host(const bsv_V2f* v, int n, float4* out) {
#pragma omp parallel for schedule(static) if (n >= kParallelGather)
	for (int i = 0; i < n; ++i) out[i] = make_float4(v[i].x[0], v[i].x[1], 0.f, 0.f);
}
void gather_f3d_host(const cvtx_F3D* const* src, int n, float4* out) {
#pragma omp parallel for schedule(static) if (n >= kParallelGather)
	for (int i = 0; i < n; ++i) {
		const cvtx_F3D* f = src[i];
		out[2 * i] = make_float4(f->start.x[0], f->start.x[1], f->start.x[2], f->strength);
		out[2 * i + 1] = make_float4(f->end.x[0], f->end.x[1], f->end.x[2], 0.f);
	}
}

// True when the measurement points are the gathered particles' coordinates,
// bit for bit: the velocity call is then the particles acting on themselves.
bool points2_are_coords(const bsv_V2f* mes, const float4* rec, int n) {
	int differ = 0;
#pragma omp parallel for schedule(static) reduction(|: differ) if (n >= kParallelGather)
	for (int i = 0; i < n; ++i) {
		const float4 q = rec[i];
		const float c[2] = {q.x, q.y};
		differ |= std::memcmp(c, mes[i].x, sizeof c) != 0;
	}
	return !differ;
}

bool points_are_coords(const bsv_V3f* mes, const float4* rec, int n) {
	int differ = 0;
#pragma omp parallel for schedule(static) reduction(|: differ) if (n >= kParallelGather)
	for (int i = 0; i < n; ++i) {
		const float4 q = rec[2 * i];
		const float c[3] = {q.x, q.y, q.z};
		differ |= std::memcmp(c, mes[i].x, sizeof c) != 0;
	}
	return !differ;
}

void fill_nan(float* out, size_t n) {
	const float q = std::numeric_limits<float>::quiet_NaN();
	for (size_t i = 0; i < n; ++i) out[i] = q;
}

// One CUDA-path call: holds the runtime lock and the active context.
class GpuJob {
 public:
	explicit GpuJob(const char* what)
		: lock_(Runtime::get().lock()), what_(what), ctx_(Runtime::get().active_context()) {}
	DeviceContext* ctx() const { return ctx_; }
	bool failed() const { return status_ != 0; }
	int status() const { return status_; }

	bool check(cudaError_t e, const char* step) {
		if (status_ != 0) return false;
		if (e == cudaSuccess) return true;
		set_error(std::string(what_) + ": " + step + ": " + cudaGetErrorString(e));
		status_ = -2;
		return false;
	}
	// Ensure pinned + device buffers of `bytes`; returns the pinned pointer.
	float4* stage(HostBuf& h, DevBuf& d, size_t bytes) {
		if (!check(h.ensure(bytes), "pinned allocation")) return nullptr;
		if (!check(d.ensure(bytes), "device allocation")) return nullptr;
		return static_cast<float4*>(h.ptr);
	}
	void upload(HostBuf& h, DevBuf& d, size_t bytes) {
		if (bytes) check(cudaMemcpyAsync(d.ptr, h.ptr, bytes, cudaMemcpyHostToDevice, ctx_->stream), "H2D copy");
	}
	// Before the first launch: reset this path's error word and wait for
	// every earlier user of the workspace (device-pointer calls included).
	bool begin() {
		return check(cudaMemsetAsync(ctx_->d_err, 0, sizeof(unsigned), ctx_->stream), "reset error word")
			&& check(cudaStreamWaitEvent(ctx_->stream, ctx_->ws_ev, 0), "workspace order");
	}
	bool ensure_out(DevBuf& d, HostBuf& h, size_t bytes) {
		return check(d.ensure(bytes), "device allocation") && check(h.ensure(bytes), "pinned allocation");
	}
	// D2H of result(s) + error word, wait, check the device error word.
	bool finish(DevBuf& d0, HostBuf& h0, size_t b0, DevBuf* d1 = nullptr, HostBuf* h1 = nullptr, size_t b1 = 0) {
		check(cudaEventRecord(ctx_->ws_ev, ctx_->stream), "workspace order");
		check(cudaMemcpyAsync(h0.ptr, d0.ptr, b0, cudaMemcpyDeviceToHost, ctx_->stream), "D2H copy");
		if (d1 && b1) check(cudaMemcpyAsync(h1->ptr, d1->ptr, b1, cudaMemcpyDeviceToHost, ctx_->stream), "D2H copy");
		check(cudaMemcpyAsync(ctx_->h_err, ctx_->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx_->stream), "D2H error word");
		check(cudaStreamSynchronize(ctx_->stream), "stream synchronize");
		if (status_ == 0 && *ctx_->h_err != 0u) {
			set_error(std::string(what_) + ": " + device_error_text(*ctx_->h_err));
			status_ = -4;
		}
		return status_ == 0;
	}

 private:
	std::lock_guard<std::recursive_mutex> lock_;
	const char* what_;
	DeviceContext* ctx_;
	int status_ = 0;
};

bool gpu_usable(const cvtx_VortFunc* k, int* reg) {
	*reg = k ? reg_from_tag(k->cl_kernel_name_ext) : -1;
	return *reg >= 0 && Runtime::get().num_enabled() > 0;
}

// P3D induced velocity and/or stretching. Targets are either points (mes) or
// particles (ind); when ind is the source pointer array itself, or the
// points are the sources' own coordinates, the source records double as
// target records (no target upload; with the stretching, the
// self-interaction form can apply).
int gpu_p3d_induce(const char* what, const cvtx_P3D** src, int n, const bsv_V3f* mes,
	const cvtx_P3D** ind, int m, bsv_V3f* vel, bsv_V3f* dvort, int reg, float sigma)
{
	GpuJob job(what);
	DeviceContext* c = job.ctx();
	if (!c) return -3;
	const size_t sb = size_t(n) * 32, ob = size_t(m) * 12;
	float4* hs = job.stage(c->h_src, c->src, sb);
	if (!hs) return job.status();
	gather_p3d_host(src, n, hs);
	const bool alias = (ind && ind == src && m == n) ||
		(!ind && m == n && n >= kSelfCheckMin && points_are_coords(mes, hs, n));
	const float4* dtgt = static_cast<const float4*>(c->src.ptr);
	int tstride = 2;
	size_t tb = 0;
	if (!alias) {
		tb = ind ? size_t(m) * 32 : size_t(m) * 16;
		float4* ht = job.stage(c->h_tgt, c->tgt, tb);
		if (!ht) return job.status();
		if (ind) gather_p3d_host(ind, m, ht);
		else pack_v3_host(mes, m, ht);
		dtgt = static_cast<const float4*>(c->tgt.ptr);
		tstride = ind ? 2 : 1;
	}
	const unsigned ops = (vel ? kOpVel : 0u) | (dvort ? kOpDvort : 0u);
	if (vel && !job.ensure_out(c->out0, c->h_out0, ob)) return job.status();
	if (dvort && !job.ensure_out(c->out1, c->h_out1, ob)) return job.status();
	P3DInduceProblem p;
	p.src = static_cast<const float4*>(c->src.ptr); p.n_src = n;
	p.tgt = alias ? p.src : dtgt; p.tstride = tstride; p.n_tgt = m;
	p.out_vel = vel ? static_cast<float*>(c->out0.ptr) : nullptr;
	p.out_dvort = dvort ? static_cast<float*>(c->out1.ptr) : nullptr;
	p.sigma = sigma;
	if (!job.check(c->ensure_ws_or(p3d_induce_ws_bytes_for(reg, ops, p, c->num_sms),
			p3d_induce_ws_bytes(reg, ops, p.n_src, p.n_tgt, c->num_sms)), "workspace"))
		return job.status();
	if (!job.begin()) return job.status();
	job.upload(c->h_src, c->src, sb);
	if (!alias) job.upload(c->h_tgt, c->tgt, tb);
	if (!job.failed()) job.check(p3d_induce(reg, ops, p, c->env()), "kernel launch");
	bool ok;
	if (vel && dvort) ok = job.finish(c->out0, c->h_out0, ob, &c->out1, &c->h_out1, ob);
	else if (vel) ok = job.finish(c->out0, c->h_out0, ob);
	else ok = job.finish(c->out1, c->h_out1, ob);
	if (!ok) return job.status();
	if (vel) std::memcpy(vel, c->h_out0.ptr, ob);
	if (dvort) std::memcpy(dvort, c->h_out1.ptr, ob);
	return 0;
}

}  // namespace
}  // namespace cvtx

using namespace cvtx;

extern "C" {

// ---- P3D (reference libcvtx.h:213-248) -----------------------------------------
CVTX_EXPORT void cvtx_P3D_M2M_vel(const cvtx_P3D** src, const int n, const bsv_V3f* mes,
	const int m, bsv_V3f* out, const cvtx_VortFunc* kernel, float sigma)
{
	if (m <= 0) return;
	int reg;
	if (!gpu_usable(kernel, &reg)) { host_P3D_M2M_vel(src, n, mes, m, out, kernel, sigma); return; }
	if (gpu_p3d_induce("cvtx_P3D_M2M_vel", src, n, mes, nullptr, m, out, nullptr, reg, sigma) != 0)
		fill_nan(&out[0].x[0], size_t(m) * 3);
}

CVTX_EXPORT void cvtx_P3D_M2M_dvort(const cvtx_P3D** src, const int n, const cvtx_P3D** ind,
	const int m, bsv_V3f* out, const cvtx_VortFunc* kernel, float sigma)
{
	if (m <= 0) return;
	int reg;
	if (!gpu_usable(kernel, &reg)) { host_P3D_M2M_dvort(src, n, ind, m, out, kernel, sigma); return; }
	if (gpu_p3d_induce("cvtx_P3D_M2M_dvort", src, n, nullptr, ind, m, nullptr, out, reg, sigma) != 0)
		fill_nan(&out[0].x[0], size_t(m) * 3);
}

CVTX_EXPORT void cvtx_P3D_M2M_visc_dvort(const cvtx_P3D** src, const int n,
	const cvtx_P3D** ind, const int m, bsv_V3f* out, const cvtx_VortFunc* kernel,
	float sigma, float nu)
{
	if (m <= 0) return;
	int reg;
	if (!gpu_usable(kernel, &reg)) {
		host_P3D_M2M_visc_dvort(src, n, ind, m, out, kernel, sigma, nu);
		return;
	}
	if (reg == 0 || reg == 2) {
		// No eta function for singular / planetary regularisation: the
		// reference (NDEBUG build) warns once and models the flow as inviscid.
		kernel->eta_3D(0.f);
		std::memset(out, 0, sizeof(bsv_V3f) * size_t(m));
		return;
	}
	GpuJob job("cvtx_P3D_M2M_visc_dvort");
	DeviceContext* c = job.ctx();
	int st = -3;
	if (c) {
		const size_t sb = size_t(n) * 32, tb = size_t(m) * 32, ob = size_t(m) * 12;
		const bool alias = ind == src && m == n;
		float4* hs = job.stage(c->h_src, c->src, sb);
		if (hs) gather_p3d_host(src, n, hs);
		float4* ht = (!alias && hs) ? job.stage(c->h_tgt, c->tgt, tb) : nullptr;
		if (ht) gather_p3d_host(ind, m, ht);
		job.ensure_out(c->out0, c->h_out0, ob);
		P3DViscProblem p;
		p.src = static_cast<const float4*>(c->src.ptr); p.n_src = n;
		p.tgt = static_cast<const float4*>(alias ? c->src.ptr : c->tgt.ptr);
		p.tstride = 2; p.n_tgt = m;
		p.out = static_cast<float*>(c->out0.ptr);
		p.sigma = sigma; p.nu = nu;
		job.check(c->ensure_ws_or(p3d_visc_ws_bytes_for(reg, p, c->num_sms),
			p3d_visc_ws_bytes(reg, n, m, c->num_sms)), "workspace");
		if (job.begin()) {
			job.upload(c->h_src, c->src, sb);
			if (!alias) job.upload(c->h_tgt, c->tgt, tb);
			job.check(p3d_visc(reg, p, c->env()), "kernel launch");
			if (job.finish(c->out0, c->h_out0, ob)) std::memcpy(out, c->h_out0.ptr, ob);
		}
		st = job.status();
	}
	if (st != 0) fill_nan(&out[0].x[0], size_t(m) * 3);
}

CVTX_EXPORT void cvtx_P3D_M2M_vort(const cvtx_P3D** src, const int n, const bsv_V3f* mes,
	const int m, bsv_V3f* out, const cvtx_VortFunc* kernel, float sigma)
{
	if (m <= 0) return;
	int reg;
	if (!gpu_usable(kernel, &reg)) { host_P3D_M2M_vort(src, n, mes, m, out, kernel, sigma); return; }
	GpuJob job("cvtx_P3D_M2M_vort");
	DeviceContext* c = job.ctx();
	int st = -3;
	if (c) {
		const size_t sb = size_t(n) * 32, tb = size_t(m) * 16, ob = size_t(m) * 12;
		float4* hs = job.stage(c->h_src, c->src, sb);
		if (hs) gather_p3d_host(src, n, hs);
		// points that are the particles' own positions bit for bit (the
		// Pedrizzetti relaxation): the records serve as targets
		const bool alias = hs && m == n && n >= kSelfCheckMin && points_are_coords(mes, hs, n);
		float4* ht = (hs && !alias) ? job.stage(c->h_tgt, c->tgt, tb) : nullptr;
		if (ht) pack_v3_host(mes, m, ht);
		job.ensure_out(c->out0, c->h_out0, ob);
		P3DVortProblem p;
		p.src = static_cast<const float4*>(c->src.ptr); p.n_src = n;
		p.tgt = static_cast<const float4*>(alias ? c->src.ptr : c->tgt.ptr);
		p.tstride = alias ? 2 : 1; p.n_tgt = m;
		p.out = static_cast<float*>(c->out0.ptr);
		p.sigma = sigma;
		job.check(c->ensure_ws_or(p3d_vort_ws_bytes_for(reg, p, c->num_sms),
			p3d_vort_ws_bytes(reg, n, m, c->num_sms)), "workspace");
		if (job.begin()) {
			job.upload(c->h_src, c->src, sb);
			if (!alias) job.upload(c->h_tgt, c->tgt, tb);
			job.check(p3d_vort(reg, p, c->env()), "kernel launch");
			if (job.finish(c->out0, c->h_out0, ob)) std::memcpy(out, c->h_out0.ptr, ob);
		}
		st = job.status();
	}
	if (st != 0) fill_nan(&out[0].x[0], size_t(m) * 3);
}

// Pedrizzetti relaxation (reference src/P3D.cpp:660-707): the vorticity field
// at the particles comes from cvtx_P3D_M2M_vort (GPU when enabled).
CVTX_EXPORT void cvtx_P3D_pedrizzetti_relaxation(cvtx_P3D** particles, const int n,
	float fdt, const cvtx_VortFunc* kernel, float sigma)
{
	if (n <= 0) return;
	bsv_V3f* mes = new bsv_V3f[n];
	bsv_V3f* om = new bsv_V3f[n];
	for (int i = 0; i < n; ++i) mes[i] = particles[i]->coord;
	cvtx_P3D_M2M_vort(const_cast<const cvtx_P3D**>(particles), n, mes, n, om, kernel, sigma);
	const float keep = 1.f - fdt;
#pragma omp parallel for
	for (int i = 0; i < n; ++i) {
		const bsv_V3f a = particles[i]->vorticity;
		const float wabs = bsv_V3f_abs(om[i]);
		const float coeff = bsv_V3f_abs(a) / wabs;
		bsv_V3f na = bsv_V3f_plus(bsv_V3f_mult(a, keep), bsv_V3f_mult(om[i], coeff * fdt));
		particles[i]->vorticity = wabs != 0.f ? na : bsv_V3f_zero();
	}
	delete[] mes;
	delete[] om;
}

// ---- P2D (reference libcvtx.h:329-370) ------------------------------------------
CVTX_EXPORT void cvtx_P2D_M2M_vel(const cvtx_P2D** src, const int n, const bsv_V2f* mes,
	const int m, bsv_V2f* out, const cvtx_VortFunc* kernel, float sigma)
{
	if (m <= 0) return;
	int reg;
	if (!gpu_usable(kernel, &reg)) { host_P2D_M2M_vel(src, n, mes, m, out, kernel, sigma); return; }
	GpuJob job("cvtx_P2D_M2M_vel");
	DeviceContext* c = job.ctx();
	int st = -3;
	if (c) {
		const size_t sb = size_t(n) * 16, tb = size_t(m) * 16, ob = size_t(m) * 8;
		float4* hs = job.stage(c->h_src, c->src, sb);
		if (hs) gather_p2d_host(src, n, hs);
		// points that are the particles' own positions bit for bit: the
		// particle records serve as targets (no upload, self-interaction form)
		const bool alias = hs && m == n && n >= kSelfCheckMin && points2_are_coords(mes, hs, n);
		float4* ht = (hs && !alias) ? job.stage(c->h_tgt, c->tgt, tb) : nullptr;
		if (ht) pack_v2_host(mes, m, ht);
		job.ensure_out(c->out0, c->h_out0, ob);
		P2DVelProblem p;
		p.src = static_cast<const float4*>(c->src.ptr); p.n_src = n;
		p.tgt = static_cast<const float4*>(alias ? c->src.ptr : c->tgt.ptr); p.n_tgt = m;
		p.out = static_cast<float*>(c->out0.ptr);
		p.sigma = sigma;
		job.check(c->ensure_ws_or(p2d_vel_ws_bytes_for(reg, p, c->num_sms),
			p2d_vel_ws_bytes(reg, n, m, c->num_sms)), "workspace");
		if (job.begin()) {
			job.upload(c->h_src, c->src, sb);
			if (!alias) job.upload(c->h_tgt, c->tgt, tb);
			job.check(p2d_vel(reg, p, c->env()), "kernel launch");
			if (job.finish(c->out0, c->h_out0, ob)) std::memcpy(out, c->h_out0.ptr, ob);
		}
		st = job.status();
	}
	if (st != 0) fill_nan(&out[0].x[0], size_t(m) * 2);
}

CVTX_EXPORT void cvtx_P2D_M2M_visc_dvort(const cvtx_P2D** src, const int n,
	const cvtx_P2D** ind, const int m, float* out, const cvtx_VortFunc* kernel,
	float sigma, float nu)
{
	if (m <= 0) return;
	int reg;
	if (!gpu_usable(kernel, &reg)) {
		host_P2D_M2M_visc_dvort(src, n, ind, m, out, kernel, sigma, nu);
		return;
	}
	if (reg == 0 || reg == 2) {
		kernel->eta_2D(0.f);
		std::memset(out, 0, sizeof(float) * size_t(m));
		return;
	}
	GpuJob job("cvtx_P2D_M2M_visc_dvort");
	DeviceContext* c = job.ctx();
	int st = -3;
	if (c) {
		const size_t sb = size_t(n) * 16, tb = size_t(m) * 16, ob = size_t(m) * 4;
		const bool alias = ind == src && m == n;
		float4* hs = job.stage(c->h_src, c->src, sb);
		if (hs) gather_p2d_host(src, n, hs);
		float4* ht = (!alias && hs) ? job.stage(c->h_tgt, c->tgt, tb) : nullptr;
		if (ht) gather_p2d_host(ind, m, ht);
		job.ensure_out(c->out0, c->h_out0, ob);
		P2DViscProblem p;
		p.src = static_cast<const float4*>(c->src.ptr); p.n_src = n;
		p.tgt = static_cast<const float4*>(alias ? c->src.ptr : c->tgt.ptr); p.n_tgt = m;
		p.out = static_cast<float*>(c->out0.ptr);
		p.sigma = sigma; p.nu = nu;
		job.check(c->ensure_ws_or(p2d_visc_ws_bytes_for(reg, p, c->num_sms),
			p2d_visc_ws_bytes(reg, n, m, c->num_sms)), "workspace");
		if (job.begin()) {
			job.upload(c->h_src, c->src, sb);
			if (!alias) job.upload(c->h_tgt, c->tgt, tb);
			job.check(p2d_visc(reg, p, c->env()), "kernel launch");
			if (job.finish(c->out0, c->h_out0, ob)) std::memcpy(out, c->h_out0.ptr, ob);
		}
		st = job.status();
	}
	if (st != 0) fill_nan(out, size_t(m));
}

// ---- F3D (reference libcvtx.h:285-305) ------------------------------------------
CVTX_EXPORT void cvtx_F3D_M2M_vel(const cvtx_F3D** fil, const int n, const bsv_V3f* mes,
	const int m, bsv_V3f* out)
{
	if (m <= 0) return;
	if (Runtime::get().num_enabled() == 0) { host_F3D_M2M_vel(fil, n, mes, m, out); return; }
	GpuJob job("cvtx_F3D_M2M_vel");
	DeviceContext* c = job.ctx();
	int st = -3;
	if (c) {
		const size_t sb = size_t(n) * 32, tb = size_t(m) * 16, ob = size_t(m) * 12;
		float4* hs = job.stage(c->h_src, c->src, sb);
		if (hs) gather_f3d_host(fil, n, hs);
		float4* ht = hs ? job.stage(c->h_tgt, c->tgt, tb) : nullptr;
		if (ht) pack_v3_host(mes, m, ht);
		job.ensure_out(c->out0, c->h_out0, ob);
		job.check(c->ensure_ws(f3d_vel_ws_bytes(n, m, c->num_sms)), "workspace");
		if (job.begin()) {
			job.upload(c->h_src, c->src, sb);
			job.upload(c->h_tgt, c->tgt, tb);
			F3DVelProblem p;
			p.fil = static_cast<const float4*>(c->src.ptr); p.n_fil = n;
			p.tgt = static_cast<const float4*>(c->tgt.ptr); p.tstride = 1; p.n_tgt = m;
			p.out = static_cast<float*>(c->out0.ptr);
			job.check(f3d_vel(p, c->env()), "kernel launch");
			if (job.finish(c->out0, c->h_out0, ob)) std::memcpy(out, c->h_out0.ptr, ob);
		}
		st = job.status();
	}
	if (st != 0) fill_nan(&out[0].x[0], size_t(m) * 3);
}

CVTX_EXPORT void cvtx_F3D_M2M_dvort(const cvtx_F3D** fil, const int n, const cvtx_P3D** ind,
	const int m, bsv_V3f* out)
{
	if (m <= 0) return;
	if (Runtime::get().num_enabled() == 0) { host_F3D_M2M_dvort(fil, n, ind, m, out); return; }
	GpuJob job("cvtx_F3D_M2M_dvort");
	DeviceContext* c = job.ctx();
	int st = -3;
	if (c) {
		const size_t sb = size_t(n) * 32, tb = size_t(m) * 32, ob = size_t(m) * 12;
		float4* hs = job.stage(c->h_src, c->src, sb);
		if (hs) gather_f3d_host(fil, n, hs);
		float4* ht = hs ? job.stage(c->h_tgt, c->tgt, tb) : nullptr;
		if (ht) gather_p3d_host(ind, m, ht);
		job.ensure_out(c->out0, c->h_out0, ob);
		job.check(c->ensure_ws(f3d_dvort_ws_bytes(n, m, c->num_sms)), "workspace");
		if (job.begin()) {
			job.upload(c->h_src, c->src, sb);
			job.upload(c->h_tgt, c->tgt, tb);
			F3DDvortProblem p;
			p.fil = static_cast<const float4*>(c->src.ptr); p.n_fil = n;
			p.tgt = static_cast<const float4*>(c->tgt.ptr); p.tstride = 2; p.n_tgt = m;
			p.out = static_cast<float*>(c->out0.ptr);
			job.check(f3d_dvort(p, c->env()), "kernel launch");
			if (job.finish(c->out0, c->h_out0, ob)) std::memcpy(out, c->h_out0.ptr, ob);
		}
		st = job.status();
	}
	if (st != 0) fill_nan(&out[0].x[0], size_t(m) * 3);
}

CVTX_EXPORT void cvtx_F3D_inf_mtrx(const cvtx_F3D** fil, const int n, const bsv_V3f* mes,
	const bsv_V3f* dir, const int m, float* out)
{
	if (m <= 0 || n <= 0) return;
	if (Runtime::get().num_enabled() == 0) { host_F3D_inf_mtrx(fil, n, mes, dir, m, out); return; }
	GpuJob job("cvtx_F3D_inf_mtrx");
	DeviceContext* c = job.ctx();
	int st = -3;
	if (c) {
		const size_t sb = size_t(n) * 32, tb = size_t(m) * 32, ob = size_t(m) * size_t(n) * 4;
		float4* hs = job.stage(c->h_src, c->src, sb);
		if (hs) gather_f3d_host(fil, n, hs);
		float4* ht = hs ? job.stage(c->h_tgt, c->tgt, tb) : nullptr;
		if (ht) { pack_v3_host(mes, m, ht); pack_v3_host(dir, m, ht + m); }
		job.ensure_out(c->out0, c->h_out0, ob);
		if (job.begin()) {
			job.upload(c->h_src, c->src, sb);
			job.upload(c->h_tgt, c->tgt, tb);
			F3DInfProblem p;
			p.fil = static_cast<const float4*>(c->src.ptr); p.n_fil = n;
			p.mes = static_cast<const float4*>(c->tgt.ptr); p.n_mes = m;
			p.dir = static_cast<const float4*>(c->tgt.ptr) + m;
			p.out = static_cast<float*>(c->out0.ptr);
			job.check(f3d_inf_mtrx(p, c->env()), "kernel launch");
			if (job.finish(c->out0, c->h_out0, ob)) std::memcpy(out, c->h_out0.ptr, ob);
		}
		st = job.status();
	}
	if (st != 0) fill_nan(out, size_t(m) * size_t(n));
}

// ---- GB300 extensions with host pointers --------------------------------------
CVTX_EXPORT int cvtx_gb300_P3D_M2M_vel_dvort(const cvtx_P3D** src, int n, bsv_V3f* vel,
	bsv_V3f* dvort, const cvtx_VortFunc* kernel, float sigma)
{
	if (n <= 0) return 0;
	if (!vel && !dvort) return 0;
	int reg;
	if (!gpu_usable(kernel, &reg)) {
		if (vel) {
			bsv_V3f* mes = new bsv_V3f[n];
			for (int i = 0; i < n; ++i) mes[i] = src[i]->coord;
			host_P3D_M2M_vel(src, n, mes, n, vel, kernel, sigma);
			delete[] mes;
		}
		if (dvort) host_P3D_M2M_dvort(src, n, src, n, dvort, kernel, sigma);
		return 0;
	}
	const int st = gpu_p3d_induce("cvtx_gb300_P3D_M2M_vel_dvort", src, n, nullptr, src, n,
		vel, dvort, reg, sigma);
	if (st != 0) {
		if (vel) fill_nan(&vel[0].x[0], size_t(n) * 3);
		if (dvort) fill_nan(&dvort[0].x[0], size_t(n) * 3);
	}
	return st;
}

}  // extern "C"
