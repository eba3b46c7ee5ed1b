// dev_api.cpp -- device-pointer extension API (cvtx_gb300_dev_*).
//
// For callers whose particles already live in GPU memory (a time-stepping
// solver, a serving loop, a framework tensor): no gather, no host copies, the
// kernels run on the caller's stream. Split-source partial sums use the
// active context's workspace; every call waits on the context's workspace
// event before its first launch and records it after its last, as the
// host-pointer calls do on the context's own stream, so that no two calls
// overlap on the workspace whatever streams they use. Device-side errors of
// these calls go to their own error word (cvtx_gb300_dev_status), which the
// host-pointer calls never reset.
#include <cstdint>
#include <string>

#include "cvortex/cvtx_gb300.h"
#include "nbody.h"
#include "runtime.h"

namespace cvtx {
namespace {

struct DevCall {
	std::lock_guard<std::recursive_mutex> lock;
	DeviceContext* ctx;
	cudaStream_t stream;
	explicit DevCall(void* s)
		: lock(Runtime::get().lock()), ctx(Runtime::get().active_context()),
		  stream(static_cast<cudaStream_t>(s)) {}

	// Serialise workspace users across streams. A call whose preferred form
	// needs more workspace than can be allocated runs in the form that fits
	// `fallback_bytes`.
	int prepare(size_t ws_bytes, const char* what, size_t fallback_bytes = SIZE_MAX) {
		if (!ctx) return -3;
		cudaError_t e = ctx->ensure_ws_or(ws_bytes, fallback_bytes);
		if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, ctx->ws_ev, 0);
		if (e != cudaSuccess) {
			set_error(std::string(what) + ": " + cudaGetErrorString(e));
			return -2;
		}
		return 0;
	}
	int done(cudaError_t e, const char* what) {
		if (e == cudaSuccess) e = cudaEventRecord(ctx->ws_ev, stream);
		if (e != cudaSuccess) {
			set_error(std::string(what) + ": " + cudaGetErrorString(e));
			return -2;
		}
		return 0;
	}
	LaunchEnv env() const {
		LaunchEnv v = ctx->env();
		v.stream = stream;
		v.err = ctx->d_err_dev;
		return v;
	}
};

bool bad_reg(int reg) { return reg < 0 || reg > 3; }

}  // namespace
}  // namespace cvtx

using namespace cvtx;

extern "C" {

CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M(const void* src, int n_src, const void* tgt,
	int tgt_stride, int n_tgt, float* vel_out, float* dvort_out, int reg, float sigma,
	void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_src < 0 || !tgt || bad_reg(reg) || (!vel_out && !dvort_out) || tgt_stride < 1)
		return -1;
	if (dvort_out && tgt_stride < 2) return -1;
	DevCall c(stream);
	const unsigned ops = (vel_out ? kOpVel : 0u) | (dvort_out ? kOpDvort : 0u);
	P3DInduceProblem p;
	p.src = static_cast<const float4*>(src); p.n_src = n_src;
	p.tgt = static_cast<const float4*>(tgt); p.tstride = tgt_stride; p.n_tgt = n_tgt;
	p.out_vel = vel_out; p.out_dvort = dvort_out; p.sigma = sigma;
	const int sms = c.ctx ? c.ctx->num_sms : 1;
	int st = c.prepare(p3d_induce_ws_bytes_for(reg, ops, p, sms), "cvtx_gb300_dev_P3D_M2M",
		p3d_induce_ws_bytes(reg, ops, n_src, n_tgt, sms));
	if (st) return st;
	return c.done(p3d_induce(reg, ops, p, c.env()), "cvtx_gb300_dev_P3D_M2M");
}

CVTX_EXPORT long long cvtx_gb300_dev_P3D_M2M_ws_bytes(int n_src, int n_tgt, int self,
	int reg, int ops, int form)
{
	if (n_src < 0 || n_tgt < 0 || bad_reg(reg) || ops < 1 || ops > 3 || (self && n_src != n_tgt))
		return -1;
	DevCall c(nullptr);
	if (!c.ctx) return -1;
	// only the pointers' equality matters to the choice of form
	static const float4 dummy[2] = {};
	P3DInduceProblem p;
	p.src = dummy; p.n_src = n_src;
	p.tgt = self ? dummy : dummy + 1; p.tstride = 2; p.n_tgt = n_tgt;
	p.out_vel = nullptr; p.out_dvort = nullptr; p.sigma = 1.f;
	const size_t b = form ? p3d_induce_ws_bytes_for(reg, unsigned(ops), p, c.ctx->num_sms)
	                      : p3d_induce_ws_bytes(reg, unsigned(ops), n_src, n_tgt, c.ctx->num_sms);
	return static_cast<long long>(b);
}

CVTX_EXPORT int cvtx_gb300_dev_P3D_step(void* rec, int n, float* vel, float* dvort, int reg,
	float sigma, float dt, void* stream)
{
	if (n <= 0) return 0;
	if (!rec || !vel || !dvort || bad_reg(reg)) return -1;
	DevCall c(stream);
	const unsigned ops = kOpVel | kOpDvort;
	float4* r = static_cast<float4*>(rec);
	P3DInduceProblem p;
	p.src = r; p.n_src = n;
	p.tgt = r; p.tstride = 2; p.n_tgt = n;
	p.out_vel = vel; p.out_dvort = dvort; p.sigma = sigma;
	const int sms = c.ctx ? c.ctx->num_sms : 1;
	int st = c.prepare(p3d_induce_ws_bytes_for(reg, ops, p, sms), "cvtx_gb300_dev_P3D_step",
		p3d_induce_ws_bytes(reg, ops, n, n, sms));
	if (st) return st;
	cudaError_t e = p3d_induce(reg, ops, p, c.env());
	if (e == cudaSuccess) e = advance_p3d(r, n, vel, dvort, dt, c.stream);
	return c.done(e, "cvtx_gb300_dev_P3D_step");
}

CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_visc(const void* src, int n_src, const void* tgt,
	int tgt_stride, int n_tgt, float* out, int reg, float sigma, float nu, void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_src < 0 || !tgt || !out || bad_reg(reg) || tgt_stride < 2) return -1;
	DevCall c(stream);
	if (reg == 0 || reg == 2) {
		if (!c.ctx) return -3;
		const cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * 3 * size_t(n_tgt), c.stream);
		return e == cudaSuccess ? 0 : -2;
	}
	P3DViscProblem p;
	p.src = static_cast<const float4*>(src); p.n_src = n_src;
	p.tgt = static_cast<const float4*>(tgt); p.tstride = tgt_stride; p.n_tgt = n_tgt;
	p.out = out; p.sigma = sigma; p.nu = nu;
	const int sms = c.ctx ? c.ctx->num_sms : 1;
	int st = c.prepare(p3d_visc_ws_bytes_for(reg, p, sms), "cvtx_gb300_dev_P3D_M2M_visc",
		p3d_visc_ws_bytes(reg, n_src, n_tgt, sms));
	if (st) return st;
	return c.done(p3d_visc(reg, p, c.env()), "cvtx_gb300_dev_P3D_M2M_visc");
}

CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_vort(const void* src, int n_src, const void* tgt,
	int tgt_stride, int n_tgt, float* out, int reg, float sigma, void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_src < 0 || !tgt || !out || bad_reg(reg) || tgt_stride < 1) return -1;
	DevCall c(stream);
	P3DVortProblem p;
	p.src = static_cast<const float4*>(src); p.n_src = n_src;
	p.tgt = static_cast<const float4*>(tgt); p.tstride = tgt_stride; p.n_tgt = n_tgt;
	p.out = out; p.sigma = sigma;
	const int sms = c.ctx ? c.ctx->num_sms : 1;
	int st = c.prepare(p3d_vort_ws_bytes_for(reg, p, sms), "cvtx_gb300_dev_P3D_M2M_vort",
		p3d_vort_ws_bytes(reg, n_src, n_tgt, sms));
	if (st) return st;
	return c.done(p3d_vort(reg, p, c.env()), "cvtx_gb300_dev_P3D_M2M_vort");
}

CVTX_EXPORT int cvtx_gb300_dev_P2D_M2M_vel(const void* src, int n_src, const void* tgt,
	int n_tgt, float* out, int reg, float sigma, void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_src < 0 || !tgt || !out || bad_reg(reg)) return -1;
	DevCall c(stream);
	P2DVelProblem p;
	p.src = static_cast<const float4*>(src); p.n_src = n_src;
	p.tgt = static_cast<const float4*>(tgt); p.n_tgt = n_tgt;
	p.out = out; p.sigma = sigma;
	const int sms = c.ctx ? c.ctx->num_sms : 1;
	int st = c.prepare(p2d_vel_ws_bytes_for(reg, p, sms), "cvtx_gb300_dev_P2D_M2M_vel",
		p2d_vel_ws_bytes(reg, n_src, n_tgt, sms));
	if (st) return st;
	return c.done(p2d_vel(reg, p, c.env()), "cvtx_gb300_dev_P2D_M2M_vel");
}

CVTX_EXPORT int cvtx_gb300_dev_P2D_M2M_visc(const void* src, int n_src, const void* tgt,
	int n_tgt, float* out, int reg, float sigma, float nu, void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_src < 0 || !tgt || !out || bad_reg(reg)) return -1;
	DevCall c(stream);
	if (reg == 0 || reg == 2) {
		if (!c.ctx) return -3;
		const cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * size_t(n_tgt), c.stream);
		return e == cudaSuccess ? 0 : -2;
	}
	P2DViscProblem p;
	p.src = static_cast<const float4*>(src); p.n_src = n_src;
	p.tgt = static_cast<const float4*>(tgt); p.n_tgt = n_tgt;
	p.out = out; p.sigma = sigma; p.nu = nu;
	const int sms = c.ctx ? c.ctx->num_sms : 1;
	int st = c.prepare(p2d_visc_ws_bytes_for(reg, p, sms), "cvtx_gb300_dev_P2D_M2M_visc",
		p2d_visc_ws_bytes(reg, n_src, n_tgt, sms));
	if (st) return st;
	return c.done(p2d_visc(reg, p, c.env()), "cvtx_gb300_dev_P2D_M2M_visc");
}

CVTX_EXPORT int cvtx_gb300_dev_F3D_M2M_vel(const void* fil, int n_fil, const void* tgt,
	int tgt_stride, int n_tgt, float* out, void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_fil < 0 || !tgt || !out || tgt_stride < 1) return -1;
	DevCall c(stream);
	int st = c.prepare(f3d_vel_ws_bytes(n_fil, n_tgt, c.ctx ? c.ctx->num_sms : 1),
		"cvtx_gb300_dev_F3D_M2M_vel");
	if (st) return st;
	F3DVelProblem p;
	p.fil = static_cast<const float4*>(fil); p.n_fil = n_fil;
	p.tgt = static_cast<const float4*>(tgt); p.tstride = tgt_stride; p.n_tgt = n_tgt;
	p.out = out;
	return c.done(f3d_vel(p, c.env()), "cvtx_gb300_dev_F3D_M2M_vel");
}

CVTX_EXPORT int cvtx_gb300_dev_F3D_M2M_dvort(const void* fil, int n_fil, const void* tgt,
	int tgt_stride, int n_tgt, float* out, void* stream)
{
	if (n_tgt <= 0) return 0;
	if (n_fil < 0 || !tgt || !out || tgt_stride < 2) return -1;
	DevCall c(stream);
	int st = c.prepare(f3d_dvort_ws_bytes(n_fil, n_tgt, c.ctx ? c.ctx->num_sms : 1),
		"cvtx_gb300_dev_F3D_M2M_dvort");
	if (st) return st;
	F3DDvortProblem p;
	p.fil = static_cast<const float4*>(fil); p.n_fil = n_fil;
	p.tgt = static_cast<const float4*>(tgt); p.tstride = tgt_stride; p.n_tgt = n_tgt;
	p.out = out;
	return c.done(f3d_dvort(p, c.env()), "cvtx_gb300_dev_F3D_M2M_dvort");
}

CVTX_EXPORT int cvtx_gb300_dev_F3D_inf_mtrx(const void* fil, int n_fil, const void* mes,
	const void* dir, int n_mes, float* out, void* stream)
{
	if (n_mes <= 0 || n_fil <= 0) return 0;
	if (!fil || !mes || !dir || !out) return -1;
	DevCall c(stream);
	if (!c.ctx) return -3;
	F3DInfProblem p;
	p.fil = static_cast<const float4*>(fil); p.n_fil = n_fil;
	p.mes = static_cast<const float4*>(mes); p.n_mes = n_mes;
	p.dir = static_cast<const float4*>(dir);
	p.out = out;
	return c.done(f3d_inf_mtrx(p, c.env()), "cvtx_gb300_dev_F3D_inf_mtrx");
}

CVTX_EXPORT int cvtx_gb300_dev_pack_P3D(const cvtx_P3D* aos, int n, void* rec, void* stream) {
	if (n < 0 || (n > 0 && (!aos || !rec))) return -1;
	return pack_p3d(aos, n, static_cast<float4*>(rec), static_cast<cudaStream_t>(stream)) ==
		cudaSuccess ? 0 : -2;
}

CVTX_EXPORT int cvtx_gb300_dev_pack_V3f(const bsv_V3f* pts, int n, void* rec, void* stream) {
	if (n < 0 || (n > 0 && (!pts || !rec))) return -1;
	return pack_v3(pts, n, static_cast<float4*>(rec), static_cast<cudaStream_t>(stream)) ==
		cudaSuccess ? 0 : -2;
}

// Synchronise `stream`, read and reset the device error word of the active
// context. Returns 0 if no device-side wait expired since the last check.
CVTX_EXPORT int cvtx_gb300_dev_status(void* stream) {
	std::lock_guard<std::recursive_mutex> g(Runtime::get().lock());
	DeviceContext* c = Runtime::get().active_context();
	if (!c) return -3;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	unsigned w = 0;
	if (cudaStreamSynchronize(s) != cudaSuccess) return -2;
	if (cudaMemcpy(&w, c->d_err_dev, sizeof w, cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
	if (cudaMemset(c->d_err_dev, 0, sizeof w) != cudaSuccess) return -2;
	if (w) {
		set_error(device_error_text(w));
		return -4;
	}
	return 0;
}

}  // extern "C"
