// abi_host.cpp -- host-side parts of the cvtx_ ABI.
//
//  * cvtx_VortFunc_* / cvtx_RedistFunc_* factories (reference
//    src/VortFunc.cpp:52-251, src/RedistFunc.cpp:35-96). The host function
//    pointers evaluate the same formulas as the reference so that callers who
//    call them directly (e.g. the reference's known-answer tests) see the same
//    values; the GPU kernels dispatch on cl_kernel_name_ext instead.
//  * single-source / single-target functions S2S, S2M, M2S (reference
//    src/P3D.cpp:74-322, src/P2D.cpp:71-231, src/F3D.cpp:34-128): host code,
//    one target at a time, FP64 accumulation as in the reference.
//  * host_* M2M loops used when the caller has disabled every accelerator
//    (the reference then uses its OpenMP path, README "Accelerators") or
//    passes a regularisation bundle whose tag names no GPU kernel (its
//    function pointers are host code and cannot run on the GPU).
#include <cmath>
#include <cstdio>
#include <cstring>

#include "cvortex/libcvtx.h"
#include "host_paths.h"
#include "redist.h"

namespace {

constexpr float kPiF = 3.14159265359f;
constexpr float kSqrt2OverPiF = 0.7978845608028654f;
constexpr float kRecipSqrt2F = 0.7071067811865475f;

float no_eta(float) {
	static int warned = 0;
	if (!warned) {
		std::fprintf(stderr, "cvortex: viscous calculation requested with a vortex "
			"regularisation that has no eta function; modelling as inviscid.\n");
		warned = 1;
	}
	return 0.f;
}

float one(float) { return 1.f; }
float zero(float) { return 0.f; }
void comb_singular(float, float* g, float* z) { *g = 1.f; *z = 0.f; }

float g3_winck(float rho) {
	const float x2 = rho * rho;
	return ((x2 + 2.5f) * rho * x2) * powf(x2 + 1.f, -2.5f);
}
float zeta3_winck(float rho) { return 7.5f * powf(rho * rho + 1.f, -3.5f); }
float eta3_winck(float rho) { return 52.5f * powf(rho * rho + 1.f, -4.5f); }
void comb_winck(float rho, float* g, float* z) { *g = g3_winck(rho); *z = zeta3_winck(rho); }
float g2_winck(float rho) {
	const float x2 = rho * rho;
	return (x2 * x2 + x2 * 2.f) / (x2 * x2 + 2.f * x2 + 1.f);
}
float eta2_winck(float rho) {
	const float a = rho * rho + 1.f;
	const float a2 = 1.f / (a * a);
	return 24.f * expf(4.f * a * (a2 * a2)) * (a2 * a2);
}

float g3_planet(float rho) { return rho < 1.f ? rho * rho * rho : 1.f; }
float zeta3_planet(float rho) { return rho < 1.f ? 3.f : 0.f; }
void comb_planet(float rho, float* g, float* z) { *g = g3_planet(rho); *z = zeta3_planet(rho); }
float g2_planet(float rho) { return rho < 1.f ? rho * rho : 1.f; }

// erf by Abramowitz & Stegun 7.1.26, g = 1 beyond rho = 6.
float g3_gauss(float rho) {
	if (rho > 6.f) return 1.f;
	const float x = rho * kRecipSqrt2F;
	const float t = 1.f / (1.f + 0.3275911f * x);
	const float t2 = t * t, t3 = t2 * t, t4 = t2 * t2, t5 = t3 * t2;
	const float e = expf(-x * x);
	const float erfv = 1.f - (0.254829592f * t - 0.284496736f * t2 + 1.421413741f * t3
		- 1.453152027f * t4 + 1.061405429f * t5) * e;
	return erfv - rho * kSqrt2OverPiF * e;
}
float zeta3_gauss(float rho) { return kSqrt2OverPiF * expf(-rho * rho * 0.5f); }
void comb_gauss(float rho, float* g, float* z) { *g = g3_gauss(rho); *z = zeta3_gauss(rho); }
float g2_gauss(float rho) { return 1.f - expf(-rho * rho * 0.5f); }
float zeta2_gauss(float rho) { return expf(-rho * rho * 0.5f); }

cvtx_VortFunc make_vf(float (*g3)(float), float (*g2)(float), float (*z3)(float),
	void (*comb)(float, float*, float*), float (*e3)(float), float (*e2)(float),
	const char* tag)
{
	cvtx_VortFunc v;
	std::memset(&v, 0, sizeof v);
	v.g_3D = g3; v.g_2D = g2; v.zeta_3D = z3; v.combined_3D = comb;
	v.eta_3D = e3; v.eta_2D = e2;
	std::strncpy(v.cl_kernel_name_ext, tag, sizeof v.cl_kernel_name_ext - 1);
	return v;
}

// Redistribution kernels (reference src/RedistFunc.cpp:35-96).
float lambda0(float u) { return u < 0.5f ? 1.f : 0.f; }
float lambda1(float u) { return u <= 1.f ? 1.f - u : 0.f; }
float lambda2(float u) {
	return u < 0.5f ? 1.f - u * u : (u < 1.5f ? 0.5f * (1.f - u) * (2.f - u) : 0.f);
}
float lambda3(float u) {
	return u < 1.f ? 0.5f * (1.f - u * u) * (2.f - u)
		: (u < 2.f ? (1.f / 6.f) * (1.f - u) * (2.f - u) * (3.f - u) : 0.f);
}
float m4p(float u) {
	return u < 1.f ? 1.f - 2.5f * u * u + 1.5f * u * u * u
		: (u < 2.f ? 0.5f * (1.f - u) * (2.f - u) * (2.f - u) : 0.f);
}
cvtx_RedistFunc make_rf(float (*f)(float), float r) {
	cvtx_RedistFunc x; x.func = f; x.radius = r; return x;
}

}  // namespace

namespace cvtx {
int redist_kind(const cvtx_RedistFunc* f) {
	if (!f) return -1;
	if (f->func == lambda0) return 0;
	if (f->func == lambda1) return 1;
	if (f->func == lambda2) return 2;
	if (f->func == lambda3) return 3;
	if (f->func == m4p) return 4;
	return -1;
}
}  // namespace cvtx

namespace {

// ---- small vector helpers --------------------------------------------------
inline bsv_V3f v3(float x, float y, float z) { bsv_V3f r = {{x, y, z}}; return r; }

}  // namespace

extern "C" {

CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_singular(void) {
	return make_vf(one, one, zero, comb_singular, no_eta, no_eta, "singular");
}
CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_winckelmans(void) {
	return make_vf(g3_winck, g2_winck, zeta3_winck, comb_winck, eta3_winck, eta2_winck,
		"winckelmans");
}
CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_planetary(void) {
	return make_vf(g3_planet, g2_planet, zeta3_planet, comb_planet, no_eta, no_eta,
		"planetary");
}
CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_gaussian(void) {
	return make_vf(g3_gauss, g2_gauss, zeta3_gauss, comb_gauss, zeta3_gauss, zeta2_gauss,
		"gaussian");
}

CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda0(void) { return make_rf(lambda0, 0.5f); }
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda1(void) { return make_rf(lambda1, 1.0f); }
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda2(void) { return make_rf(lambda2, 1.5f); }
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda3(void) { return make_rf(lambda3, 2.0f); }
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_m4p(void) { return make_rf(m4p, 2.0f); }

// ---- P3D single interactions (reference src/P3D.cpp:51-161) -----------------
// Velocity at mes from one particle, without 1/(4 pi); coincident -> zero.
static bsv_V3f p3d_vel_raw(const cvtx_P3D* s, bsv_V3f m, const cvtx_VortFunc* k, float rs) {
	if (bsv_V3f_isequal(s->coord, m)) return bsv_V3f_zero();
	const bsv_V3f d = bsv_V3f_minus(m, s->coord);
	const float r = bsv_V3f_abs(d);
	const float f = -k->g_3D(r * rs) * powf(r, -3);
	return bsv_V3f_mult(bsv_V3f_cross(d, s->vorticity), f);
}

CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_vel(const cvtx_P3D* self, const bsv_V3f mes_point,
	const cvtx_VortFunc* kernel, float regularisation_radius)
{
	const bsv_V3f v = p3d_vel_raw(self, mes_point, kernel, 1.f / fabsf(regularisation_radius));
	return bsv_V3f_mult(v, 1.f / (4.f * kPiF));
}

CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_dvort(const cvtx_P3D* self, const cvtx_P3D* ind,
	const cvtx_VortFunc* kernel, float sigma)
{
	if (bsv_V3f_isequal(self->coord, ind->coord)) return bsv_V3f_zero();
	const bsv_V3f d = bsv_V3f_minus(ind->coord, self->coord);
	const float r = bsv_V3f_abs(d);
	const float rho = fabsf(r / sigma);
	float g, z;
	kernel->combined_3D(rho, &g, &z);
	const bsv_V3f co = bsv_V3f_cross(ind->vorticity, self->vorticity);
	const float t1 = 1.f / (4.f * kPiF * powf(sigma, 3));
	const float rho3 = rho * rho * rho;
	const bsv_V3f a = bsv_V3f_div(bsv_V3f_mult(co, g), rho3);
	const float k = (-1.f / (r * r)) * ((3 * g) / rho3 - z) * bsv_V3f_dot(d, co);
	return bsv_V3f_mult(bsv_V3f_plus(a, bsv_V3f_mult(d, k)), t1);
}

CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_visc_dvort(const cvtx_P3D* self, const cvtx_P3D* ind,
	const cvtx_VortFunc* kernel, float sigma, float nu)
{
	if (bsv_V3f_isequal(self->coord, ind->coord)) return bsv_V3f_zero();
	const float r = bsv_V3f_abs(bsv_V3f_minus(self->coord, ind->coord));
	const float rho = fabsf(r / sigma);
	const float t1 = 2 * nu / powf(sigma, 2);
	const bsv_V3f w = bsv_V3f_plus(bsv_V3f_mult(self->vorticity, ind->volume),
		bsv_V3f_mult(ind->vorticity, -1 * self->volume));
	return bsv_V3f_mult(bsv_V3f_mult(w, kernel->eta_3D(rho)), t1);
}

CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_vort(const cvtx_P3D* self, const bsv_V3f mes_point,
	const cvtx_VortFunc* kernel, float sigma)
{
	const float r = bsv_V3f_abs(bsv_V3f_minus(self->coord, mes_point));
	const float c = kernel->zeta_3D(r / sigma) / (4.f * kPiF * sigma * sigma * sigma);
	return bsv_V3f_mult(self->vorticity, c);
}

CVTX_EXPORT void cvtx_P3D_S2M_vel(const cvtx_P3D* self, const bsv_V3f* mes, const int n,
	bsv_V3f* out, const cvtx_VortFunc* kernel, float sigma)
{
#pragma omp parallel for
	for (int i = 0; i < n; ++i) out[i] = cvtx_P3D_S2S_vel(self, mes[i], kernel, sigma);
}

CVTX_EXPORT void cvtx_P3D_S2M_dvort(const cvtx_P3D* self, const cvtx_P3D** ind, const int n,
	bsv_V3f* out, const cvtx_VortFunc* kernel, float sigma)
{
#pragma omp parallel for
	for (int i = 0; i < n; ++i) out[i] = cvtx_P3D_S2S_dvort(self, ind[i], kernel, sigma);
}

CVTX_EXPORT void cvtx_P3D_S2M_visc_dvort(const cvtx_P3D* self, const cvtx_P3D** ind,
	const int n, bsv_V3f* out, const cvtx_VortFunc* kernel, float sigma, float nu)
{
#pragma omp parallel for
	for (int i = 0; i < n; ++i) out[i] = cvtx_P3D_S2S_visc_dvort(self, ind[i], kernel, sigma, nu);
}

CVTX_EXPORT void cvtx_P3D_S2M_vort(const cvtx_P3D* self, const bsv_V3f* mes, const int n,
	bsv_V3f* out, const cvtx_VortFunc* kernel, float sigma)
{
#pragma omp parallel for
	for (int i = 0; i < n; ++i) out[i] = cvtx_P3D_S2S_vort(self, mes[i], kernel, sigma);
}

CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_vel(const cvtx_P3D** src, const int n, const bsv_V3f m,
	const cvtx_VortFunc* kernel, float sigma)
{
	const float rs = 1.f / fabsf(sigma);
	double x = 0., y = 0., z = 0.;
	for (long i = 0; i < n; ++i) {
		const bsv_V3f v = p3d_vel_raw(src[i], m, kernel, rs);
		x += v.x[0]; y += v.x[1]; z += v.x[2];
	}
	return bsv_V3f_mult(v3(float(x), float(y), float(z)), 1.f / (4.f * kPiF));
}

CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_dvort(const cvtx_P3D** src, const int n,
	const cvtx_P3D* ind, const cvtx_VortFunc* kernel, float sigma)
{
	double x = 0., y = 0., z = 0.;
	for (long i = 0; i < n; ++i) {
		const bsv_V3f v = cvtx_P3D_S2S_dvort(src[i], ind, kernel, sigma);
		x += v.x[0]; y += v.x[1]; z += v.x[2];
	}
	return v3(float(x), float(y), float(z));
}

CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_visc_dvort(const cvtx_P3D** src, const int n,
	const cvtx_P3D* ind, const cvtx_VortFunc* kernel, float sigma, float nu)
{
	double x = 0., y = 0., z = 0.;
	for (long i = 0; i < n; ++i) {
		const bsv_V3f v = cvtx_P3D_S2S_visc_dvort(src[i], ind, kernel, sigma, nu);
		x += v.x[0]; y += v.x[1]; z += v.x[2];
	}
	return v3(float(x), float(y), float(z));
}

// 5 sigma box cut-off as in the reference CPU path (src/P3D.cpp:298-322).
CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_vort(const cvtx_P3D** src, const int n, const bsv_V3f m,
	const cvtx_VortFunc* kernel, float sigma)
{
	const float cut = 5.f * sigma;
	const float rs = 1 / sigma;
	bsv_V3f sum = bsv_V3f_zero();
	for (long i = 0; i < n; ++i) {
		const bsv_V3f d = bsv_V3f_minus(src[i]->coord, m);
		if (fabsf(d.x[0]) < cut && fabsf(d.x[1]) < cut && fabsf(d.x[2]) < cut) {
			const float c = kernel->zeta_3D(bsv_V3f_abs(d) * rs);
			sum = bsv_V3f_plus(bsv_V3f_mult(src[i]->vorticity, c), sum);
		}
	}
	return bsv_V3f_div(sum, 4.f * kPiF * sigma * sigma * sigma);
}

// ---- F3D single interactions (reference src/F3D.cpp:34-128) -----------------
CVTX_EXPORT bsv_V3f cvtx_F3D_S2S_vel(const cvtx_F3D* self, const bsv_V3f m) {
	const float big = 3.40282346e38f;
	const bsv_V3f r1 = bsv_V3f_minus(m, self->start);
	const bsv_V3f r2 = bsv_V3f_minus(m, self->end);
	const bsv_V3f r0 = bsv_V3f_minus(r1, r2);
	const bsv_V3f c = bsv_V3f_cross(r1, r2);
	const float t1 = self->strength / (4 * kPiF * powf(bsv_V3f_abs(c), 2));
	const float t2 = bsv_V3f_dot(r1, r0) / bsv_V3f_abs(r1) - bsv_V3f_dot(r2, r0) / bsv_V3f_abs(r2);
	return (fabsf(t1) <= big && fabsf(t2) <= big) ? bsv_V3f_mult(c, t1 * t2) : bsv_V3f_zero();
}

CVTX_EXPORT bsv_V3f cvtx_F3D_S2S_dvort(const cvtx_F3D* self, const cvtx_P3D* p) {
	const bsv_V3f r1 = bsv_V3f_minus(p->coord, self->start);
	const bsv_V3f r2 = bsv_V3f_minus(p->coord, self->end);
	const bsv_V3f r0 = bsv_V3f_minus(r1, r2);
	const float t1 = self->strength / (4 * kPiF);
	const float xl = bsv_V3f_abs(bsv_V3f_cross(r1, r0));
	const bsv_V3f t211 = bsv_V3f_div(r0, -powf(xl, 2));
	const float t212 = bsv_V3f_dot(r0, r1) / bsv_V3f_abs(r1) - bsv_V3f_dot(r0, r2) / bsv_V3f_abs(r2);
	const float xl01 = bsv_V3f_abs(bsv_V3f_cross(r0, r1));
	const float t222 = xl01 / bsv_V3f_abs(r1) - xl01 / bsv_V3f_abs(r2);
	const bsv_V3f A = bsv_V3f_mult(t211, t1 * t212);
	const float B = (3.0f / bsv_V3f_abs(r0)) * t1 * t222;
	bsv_V3f ret = bsv_V3f_plus(bsv_V3f_mult(p->vorticity, B), bsv_V3f_cross(A, p->vorticity));
	if (!bsv_V3f_isequal(ret, ret) || t222 != t222 || t212 != t212) ret = bsv_V3f_zero();
	return ret;
}

CVTX_EXPORT bsv_V3f cvtx_F3D_M2S_vel(const cvtx_F3D** fil, const int n, const bsv_V3f m) {
	double x = 0., y = 0., z = 0.;
	for (long i = 0; i < n; ++i) {
		const bsv_V3f v = cvtx_F3D_S2S_vel(fil[i], m);
		x += v.x[0]; y += v.x[1]; z += v.x[2];
	}
	return v3(float(x), float(y), float(z));
}

CVTX_EXPORT bsv_V3f cvtx_F3D_M2S_dvort(const cvtx_F3D** fil, const int n, const cvtx_P3D* p) {
	double x = 0., y = 0., z = 0.;
	for (long i = 0; i < n; ++i) {
		const bsv_V3f v = cvtx_F3D_S2S_dvort(fil[i], p);
		x += v.x[0]; y += v.x[1]; z += v.x[2];
	}
	return v3(float(x), float(y), float(z));
}

// ---- P2D single interactions (reference src/P2D.cpp:49-231) -------------------
static bsv_V2f p2d_vel_raw(const cvtx_P2D* s, bsv_V2f m, const cvtx_VortFunc* k, float rs) {
	if (bsv_V2f_isequal(s->coord, m)) return bsv_V2f_zero();
	const bsv_V2f d = bsv_V2f_minus(m, s->coord);
	const float r = bsv_V2f_abs(d);
	const float g = k->g_2D(r * rs);
	bsv_V2f out;
	out.x[0] = d.x[1] * s->vorticity * g / (r * r);
	out.x[1] = -d.x[0] * s->vorticity * g / (r * r);
	return out;
}

CVTX_EXPORT bsv_V2f cvtx_P2D_S2S_vel(const cvtx_P2D* self, const bsv_V2f m,
	const cvtx_VortFunc* kernel, float sigma)
{
	return bsv_V2f_mult(p2d_vel_raw(self, m, kernel, 1.f / fabsf(sigma)), 1.f / (2.f * acosf(-1.f)));
}

CVTX_EXPORT void cvtx_P2D_S2M_vel(const cvtx_P2D* self, const bsv_V2f* mes, const int n,
	bsv_V2f* out, const cvtx_VortFunc* kernel, float sigma)
{
#pragma omp parallel for
	for (int i = 0; i < n; ++i) out[i] = cvtx_P2D_S2S_vel(self, mes[i], kernel, sigma);
}

CVTX_EXPORT bsv_V2f cvtx_P2D_M2S_vel(const cvtx_P2D** src, const int n, const bsv_V2f m,
	const cvtx_VortFunc* kernel, float sigma)
{
	const float rs = 1.f / fabsf(sigma);
	double x = 0., y = 0.;
	for (long i = 0; i < n; ++i) {
		const bsv_V2f v = p2d_vel_raw(src[i], m, kernel, rs);
		x += v.x[0]; y += v.x[1];
	}
	bsv_V2f r = {{float(x), float(y)}};
	return bsv_V2f_mult(r, 1.f / (2.f * acosf(-1.f)));
}

CVTX_EXPORT float cvtx_P2D_S2S_visc_dvort(const cvtx_P2D* self, const cvtx_P2D* ind,
	const cvtx_VortFunc* kernel, float sigma, float nu)
{
	if (bsv_V2f_isequal(self->coord, ind->coord)) return 0.f;
	const float r = bsv_V2f_abs(bsv_V2f_minus(self->coord, ind->coord));
	const float rho = fabsf(r / sigma);
	const float t1 = 2 * nu / powf(sigma, 2);
	const float w = self->vorticity * ind->area + (-ind->vorticity * self->area);
	return (w * kernel->eta_2D(rho)) * t1;
}

CVTX_EXPORT void cvtx_P2D_S2M_visc_dvort(const cvtx_P2D* self, const cvtx_P2D** ind,
	const int n, float* out, const cvtx_VortFunc* kernel, float sigma, float nu)
{
#pragma omp parallel for
	for (int i = 0; i < n; ++i) out[i] = cvtx_P2D_S2S_visc_dvort(self, ind[i], kernel, sigma, nu);
}

CVTX_EXPORT float cvtx_P2D_M2S_visc_dvort(const cvtx_P2D** src, const int n,
	const cvtx_P2D* ind, const cvtx_VortFunc* kernel, float sigma, float nu)
{
	double s = 0.;
	for (long i = 0; i < n; ++i) s += double(cvtx_P2D_S2S_visc_dvort(src[i], ind, kernel, sigma, nu));
	return float(s);
}

}  // extern "C"

// ---- host M2M loops ---------------------------------------------------------
namespace cvtx {

void host_P3D_M2M_vel(const cvtx_P3D** src, int n, const bsv_V3f* mes, int m, bsv_V3f* out,
	const cvtx_VortFunc* k, float sigma)
{
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) out[i] = cvtx_P3D_M2S_vel(src, n, mes[i], k, sigma);
}
void host_P3D_M2M_dvort(const cvtx_P3D** src, int n, const cvtx_P3D** ind, int m,
	bsv_V3f* out, const cvtx_VortFunc* k, float sigma)
{
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) out[i] = cvtx_P3D_M2S_dvort(src, n, ind[i], k, sigma);
}
void host_P3D_M2M_visc_dvort(const cvtx_P3D** src, int n, const cvtx_P3D** ind, int m,
	bsv_V3f* out, const cvtx_VortFunc* k, float sigma, float nu)
{
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) out[i] = cvtx_P3D_M2S_visc_dvort(src, n, ind[i], k, sigma, nu);
}
void host_P3D_M2M_vort(const cvtx_P3D** src, int n, const bsv_V3f* mes, int m, bsv_V3f* out,
	const cvtx_VortFunc* k, float sigma)
{
#pragma omp parallel for schedule(guided)
	for (int i = 0; i < m; ++i) out[i] = cvtx_P3D_M2S_vort(src, n, mes[i], k, sigma);
}
void host_P2D_M2M_vel(const cvtx_P2D** src, int n, const bsv_V2f* mes, int m, bsv_V2f* out,
	const cvtx_VortFunc* k, float sigma)
{
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) out[i] = cvtx_P2D_M2S_vel(src, n, mes[i], k, sigma);
}
void host_P2D_M2M_visc_dvort(const cvtx_P2D** src, int n, const cvtx_P2D** ind, int m,
	float* out, const cvtx_VortFunc* k, float sigma, float nu)
{
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) out[i] = cvtx_P2D_M2S_visc_dvort(src, n, ind[i], k, sigma, nu);
}
void host_F3D_M2M_vel(const cvtx_F3D** fil, int n, const bsv_V3f* mes, int m, bsv_V3f* out) {
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) out[i] = cvtx_F3D_M2S_vel(fil, n, mes[i]);
}
void host_F3D_M2M_dvort(const cvtx_F3D** fil, int n, const cvtx_P3D** ind, int m, bsv_V3f* out) {
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i) out[i] = cvtx_F3D_M2S_dvort(fil, n, ind[i]);
}
void host_F3D_inf_mtrx(const cvtx_F3D** fil, int n, const bsv_V3f* mes, const bsv_V3f* dir,
	int m, float* out)
{
#pragma omp parallel for schedule(static)
	for (int i = 0; i < m; ++i)
		for (int j = 0; j < n; ++j)
			out[size_t(i) * n + j] = bsv_V3f_dot(cvtx_F3D_S2S_vel(fil[j], mes[i]), dir[i]);
}

}  // namespace cvtx
