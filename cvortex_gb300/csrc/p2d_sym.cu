// p2d_sym.cu -- P2D interactions of a particle set on itself, each unordered
// pair evaluated once: the velocity at the particles' own positions and the
// viscous vorticity exchange (the rotation is in sym.cuh).
//
// For the pair (t, s), d = x_t - x_s, the reference's terms
// (src/P2D.cpp:71-81, 167-194) are related:
//   vel:   t gets Gamma_s h(r) (d_y, -d_x),  s gets Gamma_t h(r) (-d_y, d_x),
//          since d changes sign with the pair and h(r) does not;
//   visc:  t gets eta(r) (Gamma_s A_t - Gamma_t A_s), s gets the negation.
// One evaluation of h (or eta) and of d serves both particles. The record
// side of the velocity repeats the per-call kernel's arithmetic for the pair
// with its roles exchanged bit for bit (the differences negate exactly);
// only the order of the sums differs. Coincident distinct particles
// contribute nothing to each other, as in the reference.
#include <cstdint>
#include <type_traits>

#include "nbody.h"
#include "sym.cuh"

namespace cvtx {

// Regularisation constants for one regularisation distance (p3d.cu).
RegConsts make_reg_consts_host(float sigma);

namespace {

// Records of one float4 (x, y, Gamma, area), the per-call kernels' 512-record
// tiles. Unroll and resident CTAs per SM timed on a GB300 (200,000-particle
// patch, G interactions/s): Gaussian velocity 6 CTAs, unroll 8: 2,822
// (4 CTAs: 2,714; unroll 16: 2,658); Winckelmans velocity 4 CTAs, unroll
// 16: 3,551 (unroll 8: 3,496; 6 CTAs: 3,323); viscous exchange 4 CTAs,
// unroll 16: Gaussian 4,403, Winckelmans 3,114 (unroll 8: 4,335 / 3,036).
constexpr int kP2DSymTile = 512;

template <Reg R> struct HFinite2 { static constexpr bool value = true; };
template <> struct HFinite2<Reg::Singular> { static constexpr bool value = false; };

// Velocity at the particles' own positions (reference src/P2D.cpp:71-81).
template <Reg R>
struct VelSym2D {
	using Problem = P2DVelProblem;
	struct Consts { RegConsts rc; double scale; };
	static constexpr int NC = 2;
	static constexpr int kUnroll = R == Reg::Gaussian ? 8 : 16;
	static constexpr int kRec = 1, kTile = kP2DSymTile, kMinBlocks = R == Reg::Gaussian ? 6 : 4;
	static constexpr bool kOwnDiagonal = false;
	static constexpr double kPlanFactor = 16.0;   // 200k patch: 0.5 % faster than 26
	struct Tgt { float2 tx[kSymH], ty[kSymH], tg[kSymH]; };

	__device__ __forceinline__ static void load(const Problem& p, int tb, int tid, int lim,
		Tgt& g)
	{
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const int t0 = min(tb + (2 * h) * kSymNT + tid, lim - 1);
			const int t1 = min(tb + (2 * h + 1) * kSymNT + tid, lim - 1);
			const float4 q0 = p.tgt[t0], q1 = p.tgt[t1];
			g.tx[h] = make_float2(q0.x, q1.x); g.ty[h] = make_float2(q0.y, q1.y);
			g.tg[h] = make_float2(q0.z, q1.z);
		}
	}

	template <bool FULL, bool SYM>
	__device__ __forceinline__ static void step(const Consts& kc, const float4* __restrict__ r,
		bool valid, const Tgt& g, float2 (&acc)[NC][kSymH], float (&js)[NC])
	{
		float4 s = r[0];
		if (!FULL && !valid) s = make_float4(0.f, 0.f, 0.f, 0.f);
		const float2 nsx = bc2(-s.x), nsy = bc2(-s.y), gs = bc2(s.z);
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const float2 dx = __fadd2_rn(g.tx[h], nsx);
			const float2 dy = __fadd2_rn(g.ty[h], nsy);
			const float2 r2 = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
			float2 hh = RegP2D2<R>::h2(r2, kc.rc);
			if (!HFinite2<R>::value) {
				hh.x = r2.x > 0.f ? hh.x : 0.f;
				hh.y = r2.y > 0.f ? hh.y : 0.f;
			}
			if (!FULL && !valid) hh = make_float2(0.f, 0.f);
			// t: Gamma_s h (d_y, -d_x)
			const float2 hg = __fmul2_rn(hh, gs);
			acc[0][h] = __ffma2_rn(hg, dy, acc[0][h]);
			acc[1][h] = __ffma2_rn(make_float2(-hg.x, -hg.y), dx, acc[1][h]);
			if (SYM) {
				// s: Gamma_t h (-d_y, d_x)
				const float2 ht = __fmul2_rn(hh, g.tg[h]);
				js[0] = fmaf(-ht.x, dy.x, fmaf(-ht.y, dy.y, js[0]));
				js[1] = fmaf(ht.x, dx.x, fmaf(ht.y, dx.y, js[1]));
			}
		}
	}

	__device__ __forceinline__ static void write(const Problem& p, const Consts& kc, int t,
		const double* s)
	{
		p.out[2 * size_t(t)] = float(kc.scale * s[0]);
		p.out[2 * size_t(t) + 1] = float(kc.scale * s[1]);
	}
};

// Viscous exchange (PSE, reference src/P2D.cpp:167-194): the per-pair
// difference Gamma_s A_t - Gamma_t A_s formed as in the per-call kernels.
template <Reg R>
struct ViscSym2D {
	using Problem = P2DViscProblem;
	struct Consts { RegConsts rc; double scale; };
	static constexpr int NC = 1;
	static constexpr int kUnroll = 16;
	static constexpr int kRec = 1, kTile = kP2DSymTile, kMinBlocks = 4;
	static constexpr bool kOwnDiagonal = false;
	static constexpr double kPlanFactor = 16.0;   // 200k patch: 0.5 % faster than 26
	struct Tgt { float2 ntx[kSymH], nty[kSymH], ntg[kSymH], ta[kSymH]; };

	__device__ __forceinline__ static void load(const Problem& p, int tb, int tid, int lim,
		Tgt& g)
	{
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const int t0 = min(tb + (2 * h) * kSymNT + tid, lim - 1);
			const int t1 = min(tb + (2 * h + 1) * kSymNT + tid, lim - 1);
			const float4 q0 = p.tgt[t0], q1 = p.tgt[t1];
			g.ntx[h] = make_float2(-q0.x, -q1.x); g.nty[h] = make_float2(-q0.y, -q1.y);
			g.ntg[h] = make_float2(-q0.z, -q1.z); g.ta[h] = make_float2(q0.w, q1.w);
		}
	}

	template <bool FULL, bool SYM>
	__device__ __forceinline__ static void step(const Consts& kc, const float4* __restrict__ r,
		bool valid, const Tgt& g, float2 (&acc)[NC][kSymH], float (&js)[NC])
	{
		float4 s = r[0];
		if (!FULL && !valid) s = make_float4(0.f, 0.f, 0.f, 0.f);
		const float2 sx = bc2(s.x), sy = bc2(s.y), sg = bc2(s.z), sa = bc2(s.w);
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const float2 dx = __fadd2_rn(sx, g.ntx[h]);
			const float2 dy = __fadd2_rn(sy, g.nty[h]);
			const float2 r2 = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
			float2 e = RegEta2D2<R>::eta2(r2, kc.rc);
			e.x = r2.x > 0.f ? e.x : 0.f;
			e.y = r2.y > 0.f ? e.y : 0.f;
			if (!FULL && !valid) e = make_float2(0.f, 0.f);
			// Gamma_s A_t - Gamma_t A_s
			const float2 w = __ffma2_rn(sg, g.ta[h], __fmul2_rn(g.ntg[h], sa));
			acc[0][h] = __ffma2_rn(e, w, acc[0][h]);
			if (SYM) js[0] = fmaf(-e.x, w.x, fmaf(-e.y, w.y, js[0]));
		}
	}

	__device__ __forceinline__ static void write(const Problem& p, const Consts& kc, int t,
		const double* s)
	{
		p.out[t] = float(kc.scale * s[0]);
	}
};

template <class F>
auto with_reg_2d(int reg, F&& f) {
	switch (reg) {
	case 0: return f(std::integral_constant<Reg, Reg::Singular>{});
	case 1: return f(std::integral_constant<Reg, Reg::Winckelmans>{});
	case 2: return f(std::integral_constant<Reg, Reg::Planetary>{});
	default: return f(std::integral_constant<Reg, Reg::Gaussian>{});
	}
}

}  // namespace

bool p2d_vel_self_form_applies(const P2DVelProblem& p) {
	return p.tgt == p.src && p.n_tgt == p.n_src && sym_size_ok(p.n_tgt);
}

size_t p2d_vel_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap) {
	return with_reg_2d(reg, [&](auto rt) {
		return sym_ws_bytes<VelSym2D<decltype(rt)::value>>(n, num_sms, ws_cap);
	});
}

cudaError_t p2d_vel_self(int reg, const P2DVelProblem& p, const LaunchEnv& env) {
	if (reg < 0 || reg > 3) return cudaErrorInvalidValue;
	return with_reg_2d(reg, [&](auto rt) {
		using Op = VelSym2D<decltype(rt)::value>;
		const typename Op::Consts kc{make_reg_consts_host(p.sigma), p2d_vel_scale(reg, p.sigma)};
		return sym_launch<Op>(p, kc, env);
	});
}

bool p2d_visc_self_form_applies(int reg, const P2DViscProblem& p) {
	return (reg == int(Reg::Winckelmans) || reg == int(Reg::Gaussian)) && p.tgt == p.src &&
		p.n_tgt == p.n_src && sym_size_ok(p.n_tgt);
}

size_t p2d_visc_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap) {
	return reg == int(Reg::Winckelmans) ? sym_ws_bytes<ViscSym2D<Reg::Winckelmans>>(n, num_sms, ws_cap)
	                                    : sym_ws_bytes<ViscSym2D<Reg::Gaussian>>(n, num_sms, ws_cap);
}

cudaError_t p2d_visc_self(int reg, const P2DViscProblem& p, const LaunchEnv& env) {
	const double scale = 2.0 * double(p.nu) / (double(p.sigma) * double(p.sigma));
	if (reg == int(Reg::Winckelmans)) {
		const ViscSym2D<Reg::Winckelmans>::Consts kc{make_reg_consts_host(p.sigma), scale};
		return sym_launch<ViscSym2D<Reg::Winckelmans>>(p, kc, env);
	}
	if (reg == int(Reg::Gaussian)) {
		const ViscSym2D<Reg::Gaussian>::Consts kc{make_reg_consts_host(p.sigma), scale};
		return sym_launch<ViscSym2D<Reg::Gaussian>>(p, kc, env);
	}
	return cudaErrorInvalidValue;
}

}  // namespace cvtx
