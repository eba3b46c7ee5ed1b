// regfuncs.cuh -- per-pair regularisation kernels, one struct per
// regularisation, chosen at compile time by the kernel templates.
//
// Notation: d = x_target - x_source, r2 = |d|^2, rho = r/|sigma|, x2 = rho^2.
// The reference regularisation functions (src/VortFunc.cpp:64-199) are g(rho),
// zeta(rho), eta(rho); the kernels need them in these combinations:
//
//   P3D induced velocity (src/P3D.cpp:51-72):
//     u_t = S_vel * sum_s Gs * (d x alpha_s)
//   P3D vortex stretching (src/P3D.cpp:86-114), with c = d x alpha_s:
//     dalpha_t = S_dv * [ alpha_t x sum_s Gs (alpha_s - alpha_t)
//                         + K_scale * sum_s Ks (alpha_t . c) d ]
//     because d.(alpha_t x alpha_s) = -alpha_t.c and alpha_t x alpha_t = 0.
//   P3D viscous exchange (src/P3D.cpp:116-144):
//     S_visc * sum_s Es * (alpha_s V_t - alpha_t V_s)
//   P2D velocity (src/P2D.cpp:49-69): S_vel2 * sum_s Hs * Gamma_s (dy, -dx)
//   P2D viscous exchange (src/P2D.cpp:167-194):
//     S_visc2 * sum_s Es2 * (Gamma_s A_t - Gamma_t A_s)
//
// Gs, Ks, Es, Hs are computed per pair below; S_*, K_scale are per-call
// constants computed on the host (p3d.cu / p2d.cu). Coincident pairs
// (r2 == 0) are masked to zero by the callers, as the reference does.
//
// Winckelmans, rewritten with q = x2 + 1 and s = q^-1/2 (no cancellation):
//   g/rho^3 = (q + 1.5) s^5 = s^3 + 1.5 s^5,
//   (3 g/rho^3 - zeta)/rho^2 = (3 q + 7.5) s^7 = 3 s^5 (1 + 2.5 s^2)
//   (the kernels carry K/3 and fold the 3 into the per-call scale),
//   eta3 = 52.5 s^9,  g2/rho^2 = (q + 1) s^4.
// Gaussian 3D: the reference's Abramowitz & Stegun 7.1.26 erf (with g = 1 for
// rho > 6) is used for rho >= rho_c; below rho_c, where erf minus its
// leading term cancels catastrophically in FP32, the exact Taylor series of
//   G = g/rho^3 = sqrt(2/pi) sum_n (-1)^n x2^n / (2^n n! (2n+3))
//   K = (3G - zeta)/x2 = sqrt(2/pi) sum_{n>=1} (-1)^(n+1) 2n x2^(n-1)
//                                            / (2^n n! (2n+3))
// is evaluated instead (alternating, no cancellation for x2 < 1, so FP32
// Horner is accurate to a few ulp).
#pragma once
#include "common.cuh"

namespace cvtx {

// Per-call constants derived from the regularisation distance.
struct RegConsts {
	float inv_s;      // 1/|sigma|
	float inv_s2;     // 1/sigma^2
	float s2;         // sigma^2
	float inv_s3;     // 1/|sigma|^3
	float rho_c2;     // Gaussian: series below rho^2 < rho_c2
	float exp2_half;  // -0.5 * log2(e) / sigma^2   (exp(-x2/2) = 2^(r2*this))
};

enum class Reg : int { Singular = 0, Winckelmans = 1, Planetary = 2, Gaussian = 3 };

constexpr float kSqrt2OverPi = 0.7978845608028654f;
constexpr float kRecipSqrt2 = 0.7071067811865475f;

template <Reg R> struct RegP3D;

// ---- singular: g = 1, zeta = 0 ------------------------------------------
template <> struct RegP3D<Reg::Singular> {
	// Gs = 1/r^3, Ks = 1/r^5 (K_scale = 3)
	__device__ __forceinline__ static void gk(float r2, const RegConsts&, float& G, float& K) {
		const float ir = rsqrt_refined(r2);
		const float ir2 = ir * ir;
		G = ir * ir2;
		K = G * ir2;
	}
	__device__ __forceinline__ static float g(float r2, const RegConsts&) {
		const float ir = rsqrt_approx(r2);
		return ir * ir * ir;
	}
};

// ---- Winckelmans (high-order algebraic) ---------------------------------
template <> struct RegP3D<Reg::Winckelmans> {
	// Gs = (q+1.5) s^5 = s^3 + 1.5 s^5, Ks = (3q+7.5) s^7 / 3 = s^5 (1 + 2.5 s^2)
	// (q s^2 = 1; K_scale = 3/sigma^2)
	__device__ __forceinline__ static void gk(float r2, const RegConsts& c, float& G, float& K) {
		const float q = fmaf(r2, c.inv_s2, 1.f);
		const float s = rsqrt_approx(q);
		const float s2 = s * s;
		const float s3 = s2 * s;
		const float s5 = s3 * s2;
		G = fmaf(1.5f, s5, s3);
		K = s5 * fmaf(2.5f, s2, 1.f);
	}
	__device__ __forceinline__ static float g(float r2, const RegConsts& c) {
		const float q = fmaf(r2, c.inv_s2, 1.f);
		const float s = rsqrt_approx(q);
		const float s2 = s * s;
		return (s2 * s) * fmaf(1.5f, s2, 1.f);
	}
	// eta3 / 52.5 = s^9
	__device__ __forceinline__ static float eta(float r2, const RegConsts& c) {
		const float q = fmaf(r2, c.inv_s2, 1.f);
		const float s = rsqrt_approx(q);
		const float s2 = s * s;
		const float s4 = s2 * s2;
		return s4 * s4 * s;
	}
};

// ---- planetary: g = rho^3 inside the core, 1 outside --------------------
template <> struct RegP3D<Reg::Planetary> {
	// inside: Gs = 1/|sigma|^3, Ks = 0; outside: Gs = 1/r^3, Ks = 1/r^5
	// (K_scale = 3)
	__device__ __forceinline__ static void gk(float r2, const RegConsts& c, float& G, float& K) {
		const float ir = rsqrt_refined(r2);
		const float ir2 = ir * ir;
		const float ir3 = ir * ir2;
		const bool inside = r2 < c.s2;
		G = inside ? c.inv_s3 : ir3;
		K = inside ? 0.f : ir3 * ir2;
	}
	__device__ __forceinline__ static float g(float r2, const RegConsts& c) {
		const float ir = rsqrt_approx(r2);
		return r2 < c.s2 ? c.inv_s3 : ir * ir * ir;
	}
};

// ---- Gaussian -------------------------------------------------------------
struct GaussSeries {
	// sqrt(2/pi) * sum_n (-1)^n x^n / (2^n n! (2n+3)), n = 0..6
	__device__ __forceinline__ static float G(float x) {
		float p = 1.f / 691200.f;
		p = fmaf(p, x, -1.f / 49920.f);
		p = fmaf(p, x, 1.f / 4224.f);
		p = fmaf(p, x, -1.f / 432.f);
		p = fmaf(p, x, 1.f / 56.f);
		p = fmaf(p, x, -1.f / 10.f);
		p = fmaf(p, x, 1.f / 3.f);
		return kSqrt2OverPi * p;
	}
	// sqrt(2/pi) * sum_{n>=1} (-1)^(n+1) 2n x^(n-1) / (2^n n! (2n+3)), n = 1..7
	__device__ __forceinline__ static float K(float x) {
		float p = 1.f / 783360.f;     // n = 7: 14 / (2^7 7! 17)
		p = fmaf(p, x, -1.f / 57600.f);
		p = fmaf(p, x, 1.f / 4992.f);
		p = fmaf(p, x, -1.f / 528.f);
		p = fmaf(p, x, 1.f / 72.f);
		p = fmaf(p, x, -1.f / 14.f);
		p = fmaf(p, x, 1.f / 5.f);
		return kSqrt2OverPi * p;
	}
};

template <> struct RegP3D<Reg::Gaussian> {
	// Reference A&S form of g (src/VortFunc.cpp:155-176) for rho >= rho_c,
	// given rho and e = exp(-rho^2/2). In this range g = 1 - e (poly + rho
	// sqrt(2/pi)) still cancels (by ~30x at rho = 0.5), so the rounding inside
	// it matters: t and e are evaluated correctly rounded, as the reference
	// does. Perturbations of rho itself are not amplified, so rho and its
	// inverse powers come from one approximate rsqrt.
	__device__ __forceinline__ static float g_as(float rho, float e) {
		const float a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f;
		const float a4 = -1.453152027f, a5 = 1.061405429f, p = 0.3275911f;
		const float t = __frcp_rn(fmaf(p, rho * kRecipSqrt2, 1.f));
		const float poly = t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, a5, a4), a3), a2), a1);
		const float g = (1.f - poly * e) - rho * kSqrt2OverPi * e;
		return rho > 6.f ? 1.f : g;
	}
	// Gs = g/rho^3, Ks = (3 Gs - zeta)/rho^2 (K_scale = 1/sigma^2)
	__device__ __forceinline__ static void gk(float r2, const RegConsts& c, float& G, float& K) {
		const float x2 = r2 * c.inv_s2;
		if (x2 < c.rho_c2) {
			G = GaussSeries::G(x2);
			K = GaussSeries::K(x2);
		} else {
			const float s = rsqrt_approx(x2);   // 1/rho
			const float s2 = s * s;
			const float e = expf(-0.5f * x2);
			G = g_as(x2 * s, e) * (s2 * s);
			K = fmaf(3.f, G, -kSqrt2OverPi * e) * s2;
		}
	}
	__device__ __forceinline__ static float g(float r2, const RegConsts& c) {
		const float x2 = r2 * c.inv_s2;
		if (x2 < c.rho_c2) return GaussSeries::G(x2);
		const float s = rsqrt_approx(x2);
		return g_as(x2 * s, expf(-0.5f * x2)) * (s * s * s);
	}
	// eta3 / sqrt(2/pi) = exp(-x2/2)
	__device__ __forceinline__ static float eta(float r2, const RegConsts& c) {
		return exp2f(r2 * c.exp2_half);
	}
};

// ---- packed (f32x2) evaluation for two targets at once ---------------------
// Blackwell executes fma/mul/add on float2 as one instruction (two FP32 ops),
// halving the issue slots of the per-pair arithmetic. gk2 evaluates Gs, Ks
// for the two halves of r2; the default runs the scalar code per half, the
// Winckelmans specialisation stays packed except for the two rsqrt.
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }

template <Reg R> struct RegP3D2 {
	__device__ __forceinline__ static void gk2(float2 r2, const RegConsts& c, float2& G, float2& K) {
		RegP3D<R>::gk(r2.x, c, G.x, K.x);
		RegP3D<R>::gk(r2.y, c, G.y, K.y);
	}
	__device__ __forceinline__ static float2 g2(float2 r2, const RegConsts& c) {
		return make_float2(RegP3D<R>::g(r2.x, c), RegP3D<R>::g(r2.y, c));
	}
};
template <> struct RegP3D2<Reg::Winckelmans> {
	__device__ __forceinline__ static void gk2(float2 r2, const RegConsts& c, float2& G, float2& K) {
		const float2 q = __ffma2_rn(r2, bc2(c.inv_s2), bc2(1.f));
		const float2 s = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
		const float2 s2 = __fmul2_rn(s, s);
		const float2 s3 = __fmul2_rn(s2, s);
		const float2 s5 = __fmul2_rn(s3, s2);
		G = __ffma2_rn(bc2(1.5f), s5, s3);
		K = __fmul2_rn(s5, __ffma2_rn(bc2(2.5f), s2, bc2(1.f)));
	}
	__device__ __forceinline__ static float2 g2(float2 r2, const RegConsts& c) {
		const float2 q = __ffma2_rn(r2, bc2(c.inv_s2), bc2(1.f));
		const float2 s = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
		const float2 s2 = __fmul2_rn(s, s);
		return __fmul2_rn(__fmul2_rn(s2, s), __ffma2_rn(bc2(1.5f), s2, bc2(1.f)));
	}
};

// Gaussian, packed. For rho >= rho_c the reference's A&S form as in
// RegP3D<Gaussian>, with exp(-x2/2) from ex2 and t = 1/(1 + p rho/sqrt2)
// from rcp refined by one Newton step (both within a few ulp; the A&S
// formula's own error, 1.5e-7 in erf, is larger). The series branch runs only
// when some lane of the warp has a pair below rho_c (a warp vote), and then
// for both halves with a per-element select, so warps never diverge.
template <> struct RegP3D2<Reg::Gaussian> {
	static constexpr float kNegHalfLog2e = -0.72134752044448170f;   // -log2(e)/2
	__device__ __forceinline__ static float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
	// A&S branch: G (and K when want_k) for both halves of x2
	template <bool WANT_K>
	__device__ __forceinline__ static void as2(float2 x2, float2& G, float2& K) {
		const float a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f;
		const float a4 = -1.453152027f, a5 = 1.061405429f, p = 0.3275911f;
		const float2 s = make_float2(rsqrt_approx(x2.x), rsqrt_approx(x2.y));   // 1/rho
		const float2 s2 = __fmul2_rn(s, s);
		const float2 rho = __fmul2_rn(x2, s);
		const float2 ea = __fmul2_rn(x2, bc2(kNegHalfLog2e));
		const float2 e = make_float2(ex2_approx(ea.x), ex2_approx(ea.y));
		const float2 u = __ffma2_rn(rho, bc2(p * kRecipSqrt2), bc2(1.f));
		float2 t = make_float2(rcp_approx(u.x), rcp_approx(u.y));
		t = __fmul2_rn(t, __ffma2_rn(neg(u), t, bc2(2.f)));
		float2 q = __ffma2_rn(t, bc2(a5), bc2(a4));
		q = __ffma2_rn(t, q, bc2(a3));
		q = __ffma2_rn(t, q, bc2(a2));
		q = __ffma2_rn(t, q, bc2(a1));
		const float2 poly = __fmul2_rn(t, q);
		float2 g = __ffma2_rn(neg(poly), e, bc2(1.f));
		g = __ffma2_rn(neg(__fmul2_rn(rho, bc2(kSqrt2OverPi))), e, g);
		g.x = rho.x > 6.f ? 1.f : g.x;
		g.y = rho.y > 6.f ? 1.f : g.y;
		G = __fmul2_rn(g, __fmul2_rn(s2, s));
		if (WANT_K)
			K = __fmul2_rn(__ffma2_rn(bc2(3.f), G, __fmul2_rn(bc2(-kSqrt2OverPi), e)), s2);
	}
	__device__ __forceinline__ static float2 seriesG(float2 x) {
		float2 q = __ffma2_rn(x, bc2(1.f / 691200.f), bc2(-1.f / 49920.f));
		q = __ffma2_rn(q, x, bc2(1.f / 4224.f));
		q = __ffma2_rn(q, x, bc2(-1.f / 432.f));
		q = __ffma2_rn(q, x, bc2(1.f / 56.f));
		q = __ffma2_rn(q, x, bc2(-1.f / 10.f));
		q = __ffma2_rn(q, x, bc2(1.f / 3.f));
		return __fmul2_rn(bc2(kSqrt2OverPi), q);
	}
	__device__ __forceinline__ static float2 seriesK(float2 x) {
		float2 q = __ffma2_rn(x, bc2(1.f / 783360.f), bc2(-1.f / 57600.f));
		q = __ffma2_rn(q, x, bc2(1.f / 4992.f));
		q = __ffma2_rn(q, x, bc2(-1.f / 528.f));
		q = __ffma2_rn(q, x, bc2(1.f / 72.f));
		q = __ffma2_rn(q, x, bc2(-1.f / 14.f));
		q = __ffma2_rn(q, x, bc2(1.f / 5.f));
		return __fmul2_rn(bc2(kSqrt2OverPi), q);
	}
	__device__ __forceinline__ static void gk2(float2 r2, const RegConsts& c, float2& G, float2& K) {
		const float2 x2 = __fmul2_rn(r2, bc2(c.inv_s2));
		const bool sx = x2.x < c.rho_c2, sy = x2.y < c.rho_c2;
		as2<true>(x2, G, K);
		if (__any_sync(0xffffffffu, sx || sy)) {
			const float2 gs = seriesG(x2), ks = seriesK(x2);
			if (sx) { G.x = gs.x; K.x = ks.x; }
			if (sy) { G.y = gs.y; K.y = ks.y; }
		}
	}
	__device__ __forceinline__ static float2 g2(float2 r2, const RegConsts& c) {
		const float2 x2 = __fmul2_rn(r2, bc2(c.inv_s2));
		const bool sx = x2.x < c.rho_c2, sy = x2.y < c.rho_c2;
		float2 G, K;
		as2<false>(x2, G, K);
		if (__any_sync(0xffffffffu, sx || sy)) {
			const float2 gs = seriesG(x2);
			if (sx) G.x = gs.x;
			if (sy) G.y = gs.y;
		}
		return G;
	}
};

// ---- 2D ------------------------------------------------------------------
template <Reg R> struct RegP2D;

template <> struct RegP2D<Reg::Singular> {
	// Hs = 1/r^2
	__device__ __forceinline__ static float h(float r2, const RegConsts&) {
		return 1.f / r2;
	}
};
template <> struct RegP2D<Reg::Winckelmans> {
	// Hs = (q + 1)/q^2 with q = x2 + 1  (times 1/sigma^2 on the host)
	__device__ __forceinline__ static float h(float r2, const RegConsts& c) {
		const float q = fmaf(r2, c.inv_s2, 1.f);
		const float rq = 1.f / q;
		return (q + 1.f) * (rq * rq);
	}
	// eta2 = 24 exp(4/a^3) / a^4 with a = x2 + 1 (src/VortFunc.cpp:124-131)
	__device__ __forceinline__ static float eta(float r2, const RegConsts& c) {
		const float a = fmaf(r2, c.inv_s2, 1.f);
		const float ra = 1.f / a;
		const float ra2 = ra * ra;
		const float ra4 = ra2 * ra2;
		return 24.f * expf(4.f * (ra2 * ra)) * ra4;
	}
};
template <> struct RegP2D<Reg::Planetary> {
	// inside: 1/sigma^2, outside: 1/r^2
	__device__ __forceinline__ static float h(float r2, const RegConsts& c) {
		return r2 < c.s2 ? c.inv_s2 : 1.f / r2;
	}
};
template <> struct RegP2D<Reg::Gaussian> {
	// Hs = (1 - exp(-x2/2)) / x2 (times 1/sigma^2 on the host); series
	// 1/2 (1 - y/2 + y^2/6 - y^3/24 + y^4/120 - y^5/720), y = x2/2, for y < 0.1
	__device__ __forceinline__ static float h(float r2, const RegConsts& c) {
		const float x2 = r2 * c.inv_s2;
		const float y = 0.5f * x2;
		if (y < 0.1f) {
			float p = -1.f / 720.f;
			p = fmaf(p, y, 1.f / 120.f);
			p = fmaf(p, y, -1.f / 24.f);
			p = fmaf(p, y, 1.f / 6.f);
			p = fmaf(p, y, -0.5f);
			p = fmaf(p, y, 1.f);
			return 0.5f * p;
		}
		return (1.f - expf(-y)) / x2;
	}
	__device__ __forceinline__ static float eta(float r2, const RegConsts& c) {
		return exp2f(r2 * c.exp2_half);
	}
};

// Viscous weights, packed: Winckelmans s^9 (times 52.5 on the host),
// Gaussian exp(-x2/2) (times sqrt(2/pi) on the host).
template <Reg R> struct RegEta2;
template <> struct RegEta2<Reg::Winckelmans> {
	__device__ __forceinline__ static float2 eta2(float2 r2, const RegConsts& c) {
		const float2 q = __ffma2_rn(r2, bc2(c.inv_s2), bc2(1.f));
		const float2 s = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
		const float2 s2 = __fmul2_rn(s, s);
		const float2 s4 = __fmul2_rn(s2, s2);
		return __fmul2_rn(__fmul2_rn(s4, s4), s);
	}
};
template <> struct RegEta2<Reg::Gaussian> {
	__device__ __forceinline__ static float2 eta2(float2 r2, const RegConsts& c) {
		const float2 a = __fmul2_rn(r2, bc2(c.exp2_half));
		return make_float2(ex2_approx(a.x), ex2_approx(a.y));
	}
};

// 2D viscous weights, packed (RegP2D<R>::eta two at a time; exp through ex2).
template <Reg R> struct RegEta2D2;
template <> struct RegEta2D2<Reg::Winckelmans> {
	// 24 exp(4/a^3) / a^4, a = x2 + 1
	__device__ __forceinline__ static float2 eta2(float2 r2, const RegConsts& c) {
		const float2 a = __ffma2_rn(r2, bc2(c.inv_s2), bc2(1.f));
		const float2 ra = make_float2(rcp_approx(a.x), rcp_approx(a.y));
		const float2 ra1 = __fmul2_rn(ra, __ffma2_rn(make_float2(-a.x, -a.y), ra, bc2(2.f)));
		const float2 ra2 = __fmul2_rn(ra1, ra1);
		const float2 ra4 = __fmul2_rn(ra2, ra2);
		const float2 x = __fmul2_rn(__fmul2_rn(ra2, ra1), bc2(4.f * 1.4426950408889634f));
		const float2 e = make_float2(ex2_approx(x.x), ex2_approx(x.y));
		return __fmul2_rn(__fmul2_rn(bc2(24.f), e), ra4);
	}
};
template <> struct RegEta2D2<Reg::Gaussian> {
	__device__ __forceinline__ static float2 eta2(float2 r2, const RegConsts& c) {
		const float2 a = __fmul2_rn(r2, bc2(c.exp2_half));
		return make_float2(ex2_approx(a.x), ex2_approx(a.y));
	}
};

// ---- 2D, packed (two targets per f32x2 lane pair) ----------------------------
// 1/x from rcp refined by one Newton step, t (2 - x t): within an ulp.
__device__ __forceinline__ float2 rcp2(float2 x) {
	float2 t = make_float2(rcp_approx(x.x), rcp_approx(x.y));
	return __fmul2_rn(t, __ffma2_rn(make_float2(-x.x, -x.y), t, bc2(2.f)));
}

template <Reg R> struct RegP2D2;
template <> struct RegP2D2<Reg::Singular> {
	__device__ __forceinline__ static float2 h2(float2 r2, const RegConsts&) { return rcp2(r2); }
};
template <> struct RegP2D2<Reg::Winckelmans> {
	__device__ __forceinline__ static float2 h2(float2 r2, const RegConsts& c) {
		const float2 q = __ffma2_rn(r2, bc2(c.inv_s2), bc2(1.f));
		const float2 rq = rcp2(q);
		return __fmul2_rn(__fadd2_rn(q, bc2(1.f)), __fmul2_rn(rq, rq));
	}
};
template <> struct RegP2D2<Reg::Planetary> {
	__device__ __forceinline__ static float2 h2(float2 r2, const RegConsts& c) {
		const float2 o = rcp2(r2);
		return make_float2(r2.x < c.s2 ? c.inv_s2 : o.x, r2.y < c.s2 ? c.inv_s2 : o.y);
	}
};
template <> struct RegP2D2<Reg::Gaussian> {
	// (1 - exp(-y)) / x2, y = x2/2; the series of RegP2D<Gaussian> below
	// y = 0.1, evaluated when some lane of the warp needs it (warp vote)
	__device__ __forceinline__ static float2 h2(float2 r2, const RegConsts& c) {
		const float2 x2 = __fmul2_rn(r2, bc2(c.inv_s2));
		const float2 ny = __fmul2_rn(x2, bc2(-0.72134752044448170f));   // -y log2(e)
		const float2 e = make_float2(ex2_approx(ny.x), ex2_approx(ny.y));
		float2 h = __fmul2_rn(__fadd2_rn(bc2(1.f), make_float2(-e.x, -e.y)), rcp2(x2));
		const float2 y = __fmul2_rn(bc2(0.5f), x2);
		const bool sx = y.x < 0.1f, sy = y.y < 0.1f;
		if (__any_sync(0xffffffffu, sx || sy)) {
			float2 p = __ffma2_rn(y, bc2(-1.f / 720.f), bc2(1.f / 120.f));
			p = __ffma2_rn(p, y, bc2(-1.f / 24.f));
			p = __ffma2_rn(p, y, bc2(1.f / 6.f));
			p = __ffma2_rn(p, y, bc2(-0.5f));
			p = __ffma2_rn(p, y, bc2(1.f));
			p = __fmul2_rn(bc2(0.5f), p);
			if (sx) h.x = p.x;
			if (sy) h.y = p.y;
		}
		return h;
	}
};

}  // namespace cvtx
