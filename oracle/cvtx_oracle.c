/*
 * cvtx_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C restatement of the reference cvortex CPU (OpenMP) path for the
 * all-pairs M2M interactions. Only tests, the smoke check and the CPU-baseline
 * leg of the benchmark load it; the product library never links it.
 *
 * It reproduces the reference arithmetic step by step: FP32 per pair through
 * function pointers to the regularisation functions, FP64 per-target sums,
 * an OpenMP parallel loop over targets. Each function cites the reference
 * file:line it restates. Parity pin: on x86-64 with the same compiler flags
 * it reproduces the reference library (built by oracle/build_ref.sh) bit for
 * bit for every op except P2D visc_dvort, whose reference sum order depends on
 * the OpenMP thread count (reference src/P2D.cpp:225); tests check this.
 *
 * Conventions: sources and targets are passed as arrays of pointers, exactly
 * as the reference ABI takes them, so that the timed CPU baseline does the
 * same pointer chasing as the reference.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "cvortex/libcvtx.h"

#define OR_PI_F 3.14159265359f          /* reference src/P3D.cpp:47 */
#define OR_SQRT_2_OVER_PI 0.7978845608028654f   /* src/VortFunc.cpp:49 */
#define OR_RECIP_SQRT_2 0.7071067811865475f     /* src/VortFunc.cpp:50 */

/* ---- regularisation functions (reference src/VortFunc.cpp:52-199) ------- */
static int g_bad_eta_warned = 0;
static float or_bad_eta(float rho) {          /* VortFunc.cpp:52-62, NDEBUG */
	(void)rho;
	if (!g_bad_eta_warned) {
		fprintf(stderr, "oracle: viscous call with a regularisation that has "
			"no eta function; returning zero.\n");
		g_bad_eta_warned = 1;
	}
	return 0.f;
}
static float or_g_sing3(float rho) { (void)rho; return 1.f; }      /* :64-66 */
static float or_zeta_sing3(float rho) { (void)rho; return 0.f; }   /* :68-70 */
static void or_comb_sing3(float rho, float* g, float* z) {         /* :72-76 */
	(void)rho; *g = 1.f; *z = 0.f; }
static float or_g_sing2(float rho) { (void)rho; return 1.f; }      /* :78-80 */

static float or_g_winck3(float rho) {                              /* :82-90 */
	float a = rho * rho + 2.5f;
	float b = a * rho * (rho * rho);
	float c = rho * rho + 1.f;
	return b * powf(c, -2.5f);
}
static float or_zeta_winck3(float rho) {                           /* :92-99 */
	float a = rho * rho + 1.f;
	return 7.5f * powf(a, -3.5f);
}
static float or_eta_winck3(float rho) {                            /* :101-108 */
	float b = rho * rho + 1.f;
	return 52.5f * powf(b, -4.5f);
}
static void or_comb_winck3(float rho, float* g, float* z) {        /* :110-115 */
	*g = or_g_winck3(rho); *z = or_zeta_winck3(rho); }
static float or_g_winck2(float rho) {                              /* :117-122 */
	float num = (rho * rho) * (rho * rho) + (rho * rho) * 2.f;
	float den = (rho * rho) * (rho * rho) + 2.f * (rho * rho) + 1.f;
	return num / den;
}
static float or_eta_winck2(float rho) {                            /* :124-131 */
	float a = rho * rho + 1.f;
	float a2 = 1.f / (a * a);
	float c = 24.f * expf(4.f * a * (a2 * a2));
	return c * (a2 * a2);
}
static float or_g_plan3(float rho) { return rho < 1.f ? rho * rho * rho : 1.f; } /* :133-136 */
static float or_zeta_plan3(float rho) { return rho < 1.f ? 3.f : 0.f; }          /* :138-141 */
static void or_comb_plan3(float rho, float* g, float* z) {                       /* :143-148 */
	*g = or_g_plan3(rho); *z = or_zeta_plan3(rho); }
static float or_g_plan2(float rho) { return rho < 1.f ? rho * rho : 1.f; }       /* :150-153 */

static float or_g_gauss3(float rho) {                              /* :155-176 */
	/* erf by Abramowitz & Stegun 7.1.26; g = 1 beyond rho = 6. */
	if (rho > 6.f) return 1.f;
	const float a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f;
	const float a4 = -1.453152027f, a5 = 1.061405429f, p = 0.3275911f;
	float x = rho * OR_RECIP_SQRT_2;
	float t = 1.f / (1.f + p * x);
	float t2 = t * t, t3 = t2 * t, t4 = t2 * t2, t5 = t3 * t2;
	float erfv = 1.f - (a1 * t + a2 * t2 + a3 * t3 + a4 * t4 + a5 * t5)
		* expf(-x * x);
	float term2 = rho * OR_SQRT_2_OVER_PI * expf(-x * x);
	return erfv - term2;
}
static float or_zeta_gauss3(float rho) {                           /* :178-182 */
	return OR_SQRT_2_OVER_PI * expf(-rho * rho * 0.5f); }
static void or_comb_gauss3(float rho, float* g, float* z) {        /* :184-189 */
	*g = or_g_gauss3(rho); *z = or_zeta_gauss3(rho); }
static float or_g_gauss2(float rho) { return 1.f - expf(-rho * rho * 0.5f); } /* :191-194 */
static float or_zeta_gauss2(float rho) { return expf(-rho * rho * 0.5f); }    /* :196-199 */

typedef struct {
	float (*g3)(float);
	float (*g2)(float);
	float (*zeta3)(float);
	void (*comb3)(float, float*, float*);
	float (*eta3)(float);
	float (*eta2)(float);
} or_vortfunc;

/* reg ids: 0 singular, 1 winckelmans, 2 planetary, 3 gaussian
 * (factories: reference src/VortFunc.cpp:201-251). */
static or_vortfunc or_select(int reg) {
	or_vortfunc f;
	switch (reg) {
	case 0: f.g3 = or_g_sing3; f.g2 = or_g_sing2; f.zeta3 = or_zeta_sing3;
		f.comb3 = or_comb_sing3; f.eta3 = or_bad_eta; f.eta2 = or_bad_eta; break;
	case 1: f.g3 = or_g_winck3; f.g2 = or_g_winck2; f.zeta3 = or_zeta_winck3;
		f.comb3 = or_comb_winck3; f.eta3 = or_eta_winck3; f.eta2 = or_eta_winck2; break;
	case 2: f.g3 = or_g_plan3; f.g2 = or_g_plan2; f.zeta3 = or_zeta_plan3;
		f.comb3 = or_comb_plan3; f.eta3 = or_bad_eta; f.eta2 = or_bad_eta; break;
	default: f.g3 = or_g_gauss3; f.g2 = or_g_gauss2; f.zeta3 = or_zeta_gauss3;
		f.comb3 = or_comb_gauss3; f.eta3 = or_zeta_gauss3; f.eta2 = or_zeta_gauss2; break;
	}
	return f;
}

/* Scalar entry for the known-answer tests: which = 0 g3, 1 g2, 2 zeta3,
 * 3 eta3, 4 eta2. */
float oracle_regfunc(int reg, int which, float rho) {
	or_vortfunc f = or_select(reg);
	switch (which) {
	case 0: return f.g3(rho);
	case 1: return f.g2(rho);
	case 2: return f.zeta3(rho);
	case 3: return f.eta3(rho);
	default: return f.eta2(rho);
	}
}

/* Small vector helpers with the stand-in bsv semantics. */
static inline float or_dot3(const float* a, const float* b) {
	return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline float or_len3(const float* a) { return sqrtf(or_dot3(a, a)); }
static inline void or_cross3(const float* a, const float* b, float* r) {
	r[0] = a[1] * b[2] - a[2] * b[1];
	r[1] = a[2] * b[0] - a[0] * b[2];
	r[2] = a[0] * b[1] - a[1] * b[0];
}
static inline int or_eq3(const float* a, const float* b) {
	return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }

/* ---- P3D velocity (reference src/P3D.cpp:51-72, 230-251, 324-341) ------- */
void oracle_P3D_M2M_vel(const cvtx_P3D* const* src, int n_src,
	const bsv_V3f* mes, int n_mes, bsv_V3f* out, int reg, float sigma)
{
	or_vortfunc f = or_select(reg);
	const float recip = 1.f / fabsf(sigma);
	const float scale = 1.f / (4.f * OR_PI_F);
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_mes; ++i) {
		double rx = 0., ry = 0., rz = 0.;
		const float* m = mes[i].x;
		for (long j = 0; j < n_src; ++j) {
			const cvtx_P3D* s = src[j];
			if (or_eq3(s->coord.x, m)) continue;   /* coincident: zero */
			float rad[3] = {m[0] - s->coord.x[0], m[1] - s->coord.x[1],
				m[2] - s->coord.x[2]};
			float radd = or_len3(rad);
			float rho = radd * recip;
			float cor = -f.g3(rho);
			float den = powf(radd, -3);
			float num[3];
			or_cross3(rad, s->vorticity.x, num);
			float c = cor * den;
			rx += num[0] * c; ry += num[1] * c; rz += num[2] * c;
		}
		out[i].x[0] = (float)rx * scale;
		out[i].x[1] = (float)ry * scale;
		out[i].x[2] = (float)rz * scale;
	}
}

/* ---- P3D vortex stretching (reference src/P3D.cpp:86-114, 253-273,
 *      368-385). self = inducing source, induced = target. ---------------- */
static inline void or_p3d_dvort_pair(const cvtx_P3D* self,
	const cvtx_P3D* ind, const or_vortfunc* f, float sigma, float* ret)
{
	if (or_eq3(self->coord.x, ind->coord.x)) {
		ret[0] = ret[1] = ret[2] = 0.f; return; }
	float rad[3] = {ind->coord.x[0] - self->coord.x[0],
		ind->coord.x[1] - self->coord.x[1], ind->coord.x[2] - self->coord.x[2]};
	float radd = or_len3(rad);
	float rho = fabsf(radd / sigma);
	float g, z;
	f->comb3(rho, &g, &z);
	float co[3];
	or_cross3(ind->vorticity.x, self->vorticity.x, co);
	float t1 = 1.f / (4.f * OR_PI_F * powf(sigma, 3));
	float t21d = rho * rho * rho;
	float t21[3] = {co[0] * g / t21d, co[1] * g / t21d, co[2] * g / t21d};
	float t221 = -1.f / (radd * radd);
	float t222 = (3 * g) / t21d - z;
	float t223 = or_dot3(rad, co);
	float k = t221 * t222 * t223;
	for (int c = 0; c < 3; ++c)
		ret[c] = (t21[c] + rad[c] * k) * t1;
}

void oracle_P3D_M2M_dvort(const cvtx_P3D* const* src, int n_src,
	const cvtx_P3D* const* ind, int n_ind, bsv_V3f* out, int reg, float sigma)
{
	or_vortfunc f = or_select(reg);
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_ind; ++i) {
		double r[3] = {0., 0., 0.};
		for (long j = 0; j < n_src; ++j) {
			float d[3];
			or_p3d_dvort_pair(src[j], ind[i], &f, sigma, d);
			r[0] += d[0]; r[1] += d[1]; r[2] += d[2];
		}
		for (int c = 0; c < 3; ++c) out[i].x[c] = (float)r[c];
	}
}

/* ---- P3D viscous exchange (reference src/P3D.cpp:116-144, 275-296,
 *      412-430) -------------------------------------------------------- */
void oracle_P3D_M2M_visc_dvort(const cvtx_P3D* const* src, int n_src,
	const cvtx_P3D* const* ind, int n_ind, bsv_V3f* out, int reg, float sigma,
	float nu)
{
	or_vortfunc f = or_select(reg);
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_ind; ++i) {
		double r[3] = {0., 0., 0.};
		const cvtx_P3D* t = ind[i];
		for (long j = 0; j < n_src; ++j) {
			const cvtx_P3D* s = src[j];
			if (or_eq3(s->coord.x, t->coord.x)) continue;
			float rad[3] = {s->coord.x[0] - t->coord.x[0],
				s->coord.x[1] - t->coord.x[1], s->coord.x[2] - t->coord.x[2]};
			float radd = or_len3(rad);
			float rho = fabsf(radd / sigma);
			float t1 = 2 * nu / powf(sigma, 2);
			float eta = f.eta3(rho);
			for (int c = 0; c < 3; ++c) {
				float t21 = s->vorticity.x[c] * t->volume
					+ t->vorticity.x[c] * (-1 * s->volume);
				r[c] += (t21 * eta) * t1;
			}
		}
		for (int c = 0; c < 3; ++c) out[i].x[c] = (float)r[c];
	}
}

/* ---- P3D vorticity with the 5 sigma box cut-off (reference
 *      src/P3D.cpp:298-322, 458-474) -------------------------------------- */
void oracle_P3D_M2M_vort(const cvtx_P3D* const* src, int n_src,
	const bsv_V3f* mes, int n_mes, bsv_V3f* out, int reg, float sigma)
{
	or_vortfunc f = or_select(reg);
	long i;
#pragma omp parallel for schedule(guided)
	for (i = 0; i < n_mes; ++i) {
		float cutoff = 5.f * sigma;
		float rsigma = 1 / sigma;
		float sum[3] = {0.f, 0.f, 0.f};
		for (long j = 0; j < n_src; ++j) {
			const cvtx_P3D* s = src[j];
			float rad[3] = {s->coord.x[0] - mes[i].x[0],
				s->coord.x[1] - mes[i].x[1], s->coord.x[2] - mes[i].x[2]};
			if (fabsf(rad[0]) < cutoff && fabsf(rad[1]) < cutoff
				&& fabsf(rad[2]) < cutoff) {
				float coeff = f.zeta3(or_len3(rad) * rsigma);
				for (int c = 0; c < 3; ++c)
					sum[c] = s->vorticity.x[c] * coeff + sum[c];
			}
		}
		float div = 4.f * OR_PI_F * sigma * sigma * sigma;
		for (int c = 0; c < 3; ++c) out[i].x[c] = sum[c] / div;
	}
}

/* ---- P2D velocity (reference src/P2D.cpp:49-69, 99-139) ----------------- */
void oracle_P2D_M2M_vel(const cvtx_P2D* const* src, int n_src,
	const bsv_V2f* mes, int n_mes, bsv_V2f* out, int reg, float sigma)
{
	or_vortfunc f = or_select(reg);
	const float recip = 1.f / fabsf(sigma);
	const float scale = 1.f / (2.f * acosf(-1.f));
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_mes; ++i) {
		double rx = 0., ry = 0.;
		for (long j = 0; j < n_src; ++j) {
			const cvtx_P2D* s = src[j];
			if (s->coord.x[0] == mes[i].x[0] && s->coord.x[1] == mes[i].x[1])
				continue;
			float rad0 = mes[i].x[0] - s->coord.x[0];
			float rad1 = mes[i].x[1] - s->coord.x[1];
			float radd = sqrtf(rad0 * rad0 + rad1 * rad1);
			float g = f.g2(radd * recip);
			rx += rad1 * s->vorticity * g / (radd * radd);
			ry += -rad0 * s->vorticity * g / (radd * radd);
		}
		out[i].x[0] = (float)rx * scale;
		out[i].x[1] = (float)ry * scale;
	}
}

/* ---- P2D viscous exchange (reference src/P2D.cpp:167-194, 214-250). The
 * reference sums sources with an OpenMP reduction (:225); this restatement
 * sums them in index order and parallelises over targets instead. -------- */
void oracle_P2D_M2M_visc_dvort(const cvtx_P2D* const* src, int n_src,
	const cvtx_P2D* const* ind, int n_ind, float* out, int reg, float sigma,
	float nu)
{
	or_vortfunc f = or_select(reg);
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_ind; ++i) {
		double r = 0.;
		const cvtx_P2D* t = ind[i];
		for (long j = 0; j < n_src; ++j) {
			const cvtx_P2D* s = src[j];
			if (s->coord.x[0] == t->coord.x[0] && s->coord.x[1] == t->coord.x[1])
				continue;
			float rad0 = s->coord.x[0] - t->coord.x[0];
			float rad1 = s->coord.x[1] - t->coord.x[1];
			float radd = sqrtf(rad0 * rad0 + rad1 * rad1);
			float rho = fabsf(radd / sigma);
			float t1 = 2 * nu / powf(sigma, 2);
			float t21 = s->vorticity * t->area + (-t->vorticity * s->area);
			r += (double)((t21 * f.eta2(rho)) * t1);
		}
		out[i] = (float)r;
	}
}

/* ---- F3D filaments (reference src/F3D.cpp:34-54, 56-85, 87-160) -------- */
static inline void or_f3d_vel_pair(const cvtx_F3D* fl, const float* m,
	float* ret)
{
	const float big = 3.40282346e38f;
	float r1[3], r2[3], r0[3], cr[3];
	for (int c = 0; c < 3; ++c) {
		r1[c] = m[c] - fl->start.x[c];
		r2[c] = m[c] - fl->end.x[c];
		r0[c] = r1[c] - r2[c];
	}
	or_cross3(r1, r2, cr);
	float t1 = fl->strength / (4 * OR_PI_F * powf(or_len3(cr), 2));
	float t21 = or_dot3(r1, r0) / or_len3(r1);
	float t22 = or_dot3(r2, r0) / or_len3(r2);
	float t2 = t21 - t22;
	if (fabsf(t1) <= big && fabsf(t2) <= big) {
		float k = t1 * t2;
		ret[0] = cr[0] * k; ret[1] = cr[1] * k; ret[2] = cr[2] * k;
	} else {
		ret[0] = ret[1] = ret[2] = 0.f;
	}
}

void oracle_F3D_M2M_vel(const cvtx_F3D* const* fil, int n_fil,
	const bsv_V3f* mes, int n_mes, bsv_V3f* out)
{
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_mes; ++i) {
		double r[3] = {0., 0., 0.};
		for (long j = 0; j < n_fil; ++j) {
			float v[3];
			or_f3d_vel_pair(fil[j], mes[i].x, v);
			r[0] += v[0]; r[1] += v[1]; r[2] += v[2];
		}
		for (int c = 0; c < 3; ++c) out[i].x[c] = (float)r[c];
	}
}

static inline void or_f3d_dvort_pair(const cvtx_F3D* fl, const cvtx_P3D* p,
	float* ret)
{
	float r1[3], r2[3], r0[3], x10[3], x01[3];
	for (int c = 0; c < 3; ++c) {
		r1[c] = p->coord.x[c] - fl->start.x[c];
		r2[c] = p->coord.x[c] - fl->end.x[c];
		r0[c] = r1[c] - r2[c];
	}
	float t1 = fl->strength / (4 * OR_PI_F);
	or_cross3(r1, r0, x10);
	float den = -powf(or_len3(x10), 2);
	float t211[3] = {r0[0] / den, r0[1] / den, r0[2] / den};
	float t2121 = or_dot3(r0, r1) / or_len3(r1);
	float t2122 = -or_dot3(r0, r2) / or_len3(r2);
	float t221 = (float)3.0 / or_len3(r0);
	or_cross3(r0, r1, x01);
	float t2221 = or_len3(x01) / or_len3(r1);
	float t2222 = -or_len3(x01) / or_len3(r2);
	float t222 = t2221 + t2222;
	float t212 = t2121 + t2122;
	float kA = t1 * t212;
	float A[3] = {t211[0] * kA, t211[1] * kA, t211[2] * kA};
	float B = t221 * t1 * t222;
	float ax[3];
	or_cross3(A, p->vorticity.x, ax);
	for (int c = 0; c < 3; ++c) ret[c] = p->vorticity.x[c] * B + ax[c];
	if (!(ret[0] == ret[0] && ret[1] == ret[1] && ret[2] == ret[2])
		|| t222 != t222 || t212 != t212) {
		ret[0] = ret[1] = ret[2] = 0.f;
	}
}

void oracle_F3D_M2M_dvort(const cvtx_F3D* const* fil, int n_fil,
	const cvtx_P3D* const* ind, int n_ind, bsv_V3f* out)
{
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_ind; ++i) {
		double r[3] = {0., 0., 0.};
		for (long j = 0; j < n_fil; ++j) {
			float v[3];
			or_f3d_dvort_pair(fil[j], ind[i], v);
			r[0] += v[0]; r[1] += v[1]; r[2] += v[2];
		}
		for (int c = 0; c < 3; ++c) out[i].x[c] = (float)r[c];
	}
}

/* Influence matrix (reference src/F3D.cpp:204-227): row i, column j holds
 * dot(vel of filament j at mes i, dir i). */
void oracle_F3D_inf_mtrx(const cvtx_F3D* const* fil, int n_fil,
	const bsv_V3f* mes, const bsv_V3f* dir, int n_mes, float* out)
{
	long i;
#pragma omp parallel for schedule(static)
	for (i = 0; i < n_mes; ++i) {
		for (long j = 0; j < n_fil; ++j) {
			float v[3];
			or_f3d_vel_pair(fil[j], mes[i].x, v);
			out[i * (long)n_fil + j] = or_dot3(v, dir[i].x);
		}
	}
}

int oracle_num_threads(void) {
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

/* ---- FP64 exact-math evaluation (the "error vs FP64" reference) ----------
 * Same formulas as oracle/exact.py, in double precision with the C library's
 * erf, for large error reports: P3D velocity and stretching at n_tgt targets
 * from n_src sources (arrays of xyz triples), OpenMP over targets.
 * G = g/rho^3 and K = (3G - zeta)/rho^2 come from their Taylor series for
 * the Gaussian below rho = 0.5 (the closed forms cancel there). */
static void ex_gk(int reg, double rho, double* G, double* K) {
	const double x = rho * rho;
	const double sq2pi = 0.79788456080286535588;
	switch (reg) {
	case 0: *G = 1.0 / (x * rho); *K = 3.0 * *G / x; return;
	case 1: {
		const double q = x + 1.0;
		*G = (q + 1.5) * pow(q, -2.5);
		*K = (3.0 * q + 7.5) * pow(q, -3.5);
		return;
	}
	case 2:
		if (rho < 1.0) { *G = 1.0; *K = 0.0; }
		else { *G = 1.0 / (x * rho); *K = 3.0 / (x * x * rho); }
		return;
	default:
		if (rho < 0.5) {
			double g = 0.0, k = 0.0, fact = 1.0, p2 = 1.0, xn = 1.0;
			for (int n = 0; n < 16; ++n) {
				if (n > 0) { fact *= n; p2 *= 2.0; }
				g += ((n & 1) ? -1.0 : 1.0) * xn / (p2 * fact * (2 * n + 3));
				xn *= x;
			}
			fact = 1.0; p2 = 1.0; xn = 1.0;
			for (int n = 1; n < 17; ++n) {
				fact *= n; p2 *= 2.0;
				k += ((n & 1) ? 1.0 : -1.0) * 2.0 * n * xn / (p2 * fact * (2 * n + 3));
				xn *= x;
			}
			*G = sq2pi * g;
			*K = sq2pi * k;
		} else {
			const double e = exp(-0.5 * x);
			const double g = erf(rho / sqrt(2.0)) - rho * sq2pi * e;
			*G = g / (x * rho);
			*K = (3.0 * *G - sq2pi * e) / x;
		}
		return;
	}
}

void oracle_exact_P3D_vel_dvort(const double* sx, const double* sa, int n_src,
	const double* tx, const double* ta, int n_tgt, int reg, double sigma,
	double* vel, double* dvort)
{
	const double pi = 3.14159265358979323846;
	const double as = fabs(sigma);
	long i;
#pragma omp parallel for schedule(dynamic, 16)
	for (i = 0; i < n_tgt; ++i) {
		double v[3] = {0, 0, 0}, w[3] = {0, 0, 0};
		const double* t = tx + 3 * i;
		const double* at = ta ? ta + 3 * i : 0;
		for (long j = 0; j < n_src; ++j) {
			const double* s = sx + 3 * j;
			const double* a = sa + 3 * j;
			const double d[3] = {t[0] - s[0], t[1] - s[1], t[2] - s[2]};
			const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
			if (r2 == 0.0) continue;
			double G, K;
			ex_gk(reg, sqrt(r2) / as, &G, &K);
			if (vel) {
				const double c[3] = {d[1] * a[2] - d[2] * a[1], d[2] * a[0] - d[0] * a[2],
					d[0] * a[1] - d[1] * a[0]};
				for (int k = 0; k < 3; ++k) v[k] += G * c[k];
			}
			if (dvort && at) {
				const double co[3] = {at[1] * a[2] - at[2] * a[1], at[2] * a[0] - at[0] * a[2],
					at[0] * a[1] - at[1] * a[0]};
				const double dco = d[0] * co[0] + d[1] * co[1] + d[2] * co[2];
				for (int k = 0; k < 3; ++k)
					w[k] += G * co[k] - K * dco * d[k] / (sigma * sigma);
			}
		}
		if (vel) for (int k = 0; k < 3; ++k) vel[3 * i + k] = -v[k] / (4 * pi * as * as * as);
		if (dvort) for (int k = 0; k < 3; ++k) dvort[3 * i + k] = w[k] / (4 * pi * sigma * sigma * sigma);
	}
}

/* ---- FP64 exact-math evaluation of the other ops (same formulas as
 * oracle/exact.py, in double precision). Inputs are double arrays: xyz
 * triples (or xy pairs) and per-particle scalars; OpenMP over targets.
 * Coincident pairs contribute zero, as in the reference. */

/* eta_3D(rho) (reference src/VortFunc.cpp:101-108, 178-182): Winckelmans
 * 52.5 (1 + rho^2)^-4.5, Gaussian sqrt(2/pi) exp(-rho^2/2); 0 otherwise. */
static double ex_eta3(int reg, double rho) {
	const double x = rho * rho;
	if (reg == 1) return 52.5 * pow(x + 1.0, -4.5);
	if (reg == 3) return 0.79788456080286535588 * exp(-0.5 * x);
	return 0.0;
}

/* zeta_3D(rho) (reference src/VortFunc.cpp:92-99, 138-141, 178-182). */
static double ex_zeta3(int reg, double rho) {
	const double x = rho * rho;
	switch (reg) {
	case 1: return 7.5 * pow(x + 1.0, -3.5);
	case 2: return rho < 1.0 ? 3.0 : 0.0;
	case 3: return 0.79788456080286535588 * exp(-0.5 * x);
	default: return 0.0;
	}
}

/* g_2D(rho) / r^2 (reference src/VortFunc.cpp:78-80, 117-122, 150-153,
 * 191-194), the Gaussian through expm1 (no cancellation at small rho). */
static double ex_g2_over_r2(int reg, double r2, double sigma) {
	const double s2 = sigma * sigma, x = r2 / s2;
	switch (reg) {
	case 0: return 1.0 / r2;
	case 1: return (x + 2.0) / ((x + 1.0) * (x + 1.0) * s2);
	case 2: return x < 1.0 ? 1.0 / s2 : 1.0 / r2;
	default: return -expm1(-0.5 * x) / r2;
	}
}

/* eta_2D(rho) (reference src/VortFunc.cpp:124-131, 196-199), including the
 * reference's Winckelmans form 24 exp(4/a^3)/a^4, a = 1 + rho^2. */
static double ex_eta2(int reg, double rho) {
	const double x = rho * rho;
	if (reg == 1) { const double a = x + 1.0; return 24.0 * exp(4.0 / (a * a * a)) / (a * a * a * a); }
	if (reg == 3) return exp(-0.5 * x);
	return 0.0;
}

/* P3D viscous exchange (reference src/P3D.cpp:116-144):
 * (2 nu / sigma^2) sum_s (alpha_s V_t - alpha_t V_s) eta(rho). */
void oracle_exact_P3D_visc(const double* sx, const double* sa, const double* sv, int n_src,
	const double* tx, const double* ta, const double* tv, int n_tgt, int reg, double sigma,
	double nu, double* out)
{
	const double as = fabs(sigma);
	long i;
#pragma omp parallel for schedule(dynamic, 16)
	for (i = 0; i < n_tgt; ++i) {
		double w[3] = {0, 0, 0}, vsum = 0.0;
		const double* t = tx + 3 * i;
		for (long j = 0; j < n_src; ++j) {
			const double* s = sx + 3 * j;
			const double d[3] = {s[0] - t[0], s[1] - t[1], s[2] - t[2]};
			const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
			if (r2 == 0.0) continue;
			const double e = ex_eta3(reg, sqrt(r2) / as);
			for (int k = 0; k < 3; ++k) w[k] += e * sa[3 * j + k];
			vsum += e * sv[j];
		}
		for (int k = 0; k < 3; ++k)
			out[3 * i + k] = (w[k] * tv[i] - ta[3 * i + k] * vsum) * (2.0 * nu / (sigma * sigma));
	}
}

/* P3D vorticity field with the CPU path's 5 sigma box (reference
 * src/P3D.cpp:298-322): sum_s alpha_s zeta(rho) / (4 pi sigma^3) over
 * sources with every |d_k| < 5 sigma. */
void oracle_exact_P3D_vort(const double* sx, const double* sa, int n_src,
	const double* tx, int n_tgt, int reg, double sigma, double* out)
{
	const double pi = 3.14159265358979323846;
	const double cut = 5.0 * sigma;
	long i;
#pragma omp parallel for schedule(dynamic, 16)
	for (i = 0; i < n_tgt; ++i) {
		double w[3] = {0, 0, 0};
		const double* t = tx + 3 * i;
		for (long j = 0; j < n_src; ++j) {
			const double* s = sx + 3 * j;
			const double d[3] = {s[0] - t[0], s[1] - t[1], s[2] - t[2]};
			if (!(fabs(d[0]) < cut && fabs(d[1]) < cut && fabs(d[2]) < cut)) continue;
			const double z = ex_zeta3(reg, sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / sigma);
			for (int k = 0; k < 3; ++k) w[k] += z * sa[3 * j + k];
		}
		for (int k = 0; k < 3; ++k) out[3 * i + k] = w[k] / (4.0 * pi * sigma * sigma * sigma);
	}
}

/* P2D velocity (reference src/P2D.cpp:49-69):
 * (1/2pi) sum_s Gamma_s g(rho)/r^2 (dy, -dx), d = x_t - x_s. */
void oracle_exact_P2D_vel(const double* sx, const double* sg, int n_src,
	const double* tx, int n_tgt, int reg, double sigma, double* out)
{
	const double pi = 3.14159265358979323846;
	const double as = fabs(sigma);
	long i;
#pragma omp parallel for schedule(dynamic, 16)
	for (i = 0; i < n_tgt; ++i) {
		double u = 0.0, v = 0.0;
		for (long j = 0; j < n_src; ++j) {
			const double dx = tx[2 * i] - sx[2 * j], dy = tx[2 * i + 1] - sx[2 * j + 1];
			const double r2 = dx * dx + dy * dy;
			if (r2 == 0.0) continue;
			const double h = sg[j] * ex_g2_over_r2(reg, r2, as);
			u += h * dy;
			v -= h * dx;
		}
		out[2 * i] = u / (2.0 * pi);
		out[2 * i + 1] = v / (2.0 * pi);
	}
}

/* P2D viscous exchange (reference src/P2D.cpp:167-194):
 * (2 nu / sigma^2) sum_s (Gamma_s A_t - Gamma_t A_s) eta(rho). */
void oracle_exact_P2D_visc(const double* sx, const double* sg, const double* sa, int n_src,
	const double* tx, const double* tg, const double* ta, int n_tgt, int reg, double sigma,
	double nu, double* out)
{
	const double as = fabs(sigma);
	long i;
#pragma omp parallel for schedule(dynamic, 16)
	for (i = 0; i < n_tgt; ++i) {
		double gs = 0.0, ar = 0.0;
		for (long j = 0; j < n_src; ++j) {
			const double dx = sx[2 * j] - tx[2 * i], dy = sx[2 * j + 1] - tx[2 * i + 1];
			const double r2 = dx * dx + dy * dy;
			if (r2 == 0.0) continue;
			const double e = ex_eta2(reg, sqrt(r2) / as);
			gs += e * sg[j];
			ar += e * sa[j];
		}
		out[i] = (gs * ta[i] - tg[i] * ar) * (2.0 * nu / (sigma * sigma));
	}
}

/* F3D velocity (reference src/F3D.cpp:34-54): straight-segment Biot-Savart,
 * non-finite terms dropped. */
static void ex_f3d_vel_pair(const double* a, const double* b, double g, const double* m,
	double* v)
{
	const double pi = 3.14159265358979323846;
	double r1[3], r2[3], r0[3];
	for (int k = 0; k < 3; ++k) { r1[k] = m[k] - a[k]; r2[k] = m[k] - b[k]; r0[k] = r1[k] - r2[k]; }
	const double c[3] = {r1[1] * r2[2] - r1[2] * r2[1], r1[2] * r2[0] - r1[0] * r2[2],
		r1[0] * r2[1] - r1[1] * r2[0]};
	const double cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
	const double l1 = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
	const double l2 = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
	const double t2 = (r1[0] * r0[0] + r1[1] * r0[1] + r1[2] * r0[2]) / l1
		- (r2[0] * r0[0] + r2[1] * r0[1] + r2[2] * r0[2]) / l2;
	const double f = g / (4.0 * pi * cc) * t2;
	for (int k = 0; k < 3; ++k) v[k] = isfinite(f) ? f * c[k] : 0.0;
}

/* fa, fb: filament start and end xyz; fg: strengths; dirs (optional): when
 * given, out[i * n_fil + j] = dot(vel of filament j at point i, dirs[i])
 * (the influence matrix, reference src/F3D.cpp:204-227), else out holds
 * the summed velocity per point. */
void oracle_exact_F3D_vel(const double* fa, const double* fb, const double* fg, int n_fil,
	const double* tx, const double* dirs, int n_tgt, double* out)
{
	long i;
#pragma omp parallel for schedule(dynamic, 16)
	for (i = 0; i < n_tgt; ++i) {
		double u[3] = {0, 0, 0};
		for (long j = 0; j < n_fil; ++j) {
			double v[3];
			ex_f3d_vel_pair(fa + 3 * j, fb + 3 * j, fg[j], tx + 3 * i, v);
			if (dirs) {
				const double* dd = dirs + 3 * i;
				out[i * (long)n_fil + j] = v[0] * dd[0] + v[1] * dd[1] + v[2] * dd[2];
			} else {
				for (int k = 0; k < 3; ++k) u[k] += v[k];
			}
		}
		if (!dirs) for (int k = 0; k < 3; ++k) out[3 * i + k] = u[k];
	}
}

/* F3D vortex stretching (reference src/F3D.cpp:56-85): B alpha + A x alpha
 * with A = -(gamma/4pi) r0 / |r1 x r0|^2 (r0.r1/|r1| - r0.r2/|r2|) and
 * B = (3/|r0|)(gamma/4pi) |r0 x r1| (1/|r1| - 1/|r2|); non-finite terms
 * dropped. */
void oracle_exact_F3D_dvort(const double* fa, const double* fb, const double* fg, int n_fil,
	const double* tx, const double* ta, int n_tgt, double* out)
{
	const double pi = 3.14159265358979323846;
	long i;
#pragma omp parallel for schedule(dynamic, 16)
	for (i = 0; i < n_tgt; ++i) {
		double u[3] = {0, 0, 0};
		const double* p = tx + 3 * i;
		const double* w = ta + 3 * i;
		for (long j = 0; j < n_fil; ++j) {
			const double* a = fa + 3 * j;
			const double* b = fb + 3 * j;
			double r1[3], r2[3], r0[3];
			for (int k = 0; k < 3; ++k) { r1[k] = p[k] - a[k]; r2[k] = p[k] - b[k]; r0[k] = r1[k] - r2[k]; }
			const double X[3] = {r1[1] * r0[2] - r1[2] * r0[1], r1[2] * r0[0] - r1[0] * r0[2],
				r1[0] * r0[1] - r1[1] * r0[0]};
			const double X2 = X[0] * X[0] + X[1] * X[1] + X[2] * X[2];
			const double l1 = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
			const double l2 = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
			const double l0 = sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
			const double t1 = fg[j] / (4.0 * pi);
			const double t212 = (r0[0] * r1[0] + r0[1] * r1[1] + r0[2] * r1[2]) / l1
				- (r0[0] * r2[0] + r0[1] * r2[1] + r0[2] * r2[2]) / l2;
			const double t222 = sqrt(X2) / l1 - sqrt(X2) / l2;
			const double kA = -t1 * t212 / X2;
			const double A[3] = {r0[0] * kA, r0[1] * kA, r0[2] * kA};
			const double B = 3.0 / l0 * t1 * t222;
			const double v[3] = {w[0] * B + A[1] * w[2] - A[2] * w[1],
				w[1] * B + A[2] * w[0] - A[0] * w[2], w[2] * B + A[0] * w[1] - A[1] * w[0]};
			if (isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))
				for (int k = 0; k < 3; ++k) u[k] += v[k];
		}
		for (int k = 0; k < 3; ++k) out[3 * i + k] = u[k];
	}
}
