// p3d_sym.cu -- P3D interactions of a particle set on itself, each unordered
// pair evaluated once: the velocity and / or the vortex stretching, the
// viscous vorticity exchange and the vorticity field.
//
// The all-pairs calls of the reference (src/P3D.cpp:343-366, 387-410,
// 432-456) are most often made with the particles as their own targets (a
// vortex-particle time step; the reference's benchmark,
// bench/benchP3D.c:338-345). For such a call the terms of the pair (t, s)
// that the two particles receive are related (d = x_t - x_s; p3d_induce.cuh
// gives the sums):
//   vel:   t gets G d x alpha_s,            s gets -G d x alpha_t
//   dvort: t gets G co + K (d.co) d,        s gets the negation,
//          since co = alpha_t x alpha_s changes sign with the pair and d.co
//          does not
//   visc:  t gets eta (alpha_s V_t - alpha_t V_s), s gets the negation.
// One evaluation of the pair's weights (and of co, d.co, the viscous
// difference) thus serves both particles.
//
// The rotation that evaluates each unordered pair once is in sym.cuh; the
// diagonal blocks of the induced velocity / stretching run the per-call CTA
// body (p3d_induce.cuh). Coincident distinct particles contribute nothing to
// each other, as in the reference.
#include <cstdint>
#include <type_traits>

#include "nbody.h"
#include "p3d_induce.cuh"
#include "p3d_sym_batch.h"
#include "sym.cuh"

namespace cvtx {

// Regularisation constants for one regularisation distance (p3d.cu).
RegConsts make_reg_consts_host(float sigma);

namespace {

// Resident CTAs per SM the registers are sized for (about 165 registers for
// the fused pair). Sizing for two (217 registers) measured 5-7 % slower, and
// four for one output alone (128 registers, small spills) 1-3 % slower.
constexpr int kP3DSymMinBlocks = 3;

// ---- pair operations (the interface is described in sym.cuh) --------------

// Induced velocity and/or stretching (reference src/P3D.cpp:51-114).
template <Reg R, bool VEL, bool DV>
struct InduceSym {
	using Problem = P3DInduceProblem;
	using Consts = InduceConsts;
	static constexpr int NC = InduceNC<VEL, DV>::value;
	// 1M cube, G/s: fused 8 -> 1,079, 4 -> 1,068, 2 -> 1,055; velocity /
	// stretching alone 8 -> 2,162 / 1,590, 4 -> 2,113 / 1,555, 16 -> 2,134 / 1,585
	static constexpr int kUnroll = 8;
	static constexpr int kRec = 2, kTile = kP3DTile, kMinBlocks = kP3DSymMinBlocks;
	static constexpr double kPlanFactor = 26.0;
	static constexpr bool kOwnDiagonal = true;
	struct Tgt {
		float2 tx[kSymH], ty[kSymH], tz[kSymH], ax[kSymH], ay[kSymH], az[kSymH];
		float2 nax[kSymH], nay[kSymH], naz[kSymH];
	};

	__device__ __forceinline__ static void load(const Problem& p, int tb, int tid, int lim,
		Tgt& g)
	{
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const int t0 = min(tb + (2 * h) * kSymNT + tid, lim - 1);
			const int t1 = min(tb + (2 * h + 1) * kSymNT + tid, lim - 1);
			const float4 q0 = p.tgt[2 * size_t(t0)], q1 = p.tgt[2 * size_t(t1)];
			const float4 v0 = p.tgt[2 * size_t(t0) + 1], v1 = p.tgt[2 * size_t(t1) + 1];
			g.tx[h] = make_float2(q0.x, q1.x); g.ty[h] = make_float2(q0.y, q1.y);
			g.tz[h] = make_float2(q0.z, q1.z);
			g.ax[h] = make_float2(v0.x, v1.x); g.ay[h] = make_float2(v0.y, v1.y);
			g.az[h] = make_float2(v0.z, v1.z);
			g.nax[h] = make_float2(-v0.x, -v1.x); g.nay[h] = make_float2(-v0.y, -v1.y);
			g.naz[h] = make_float2(-v0.z, -v1.z);
		}
	}

	template <bool FULL, bool SYM>
	__device__ __forceinline__ static void step(const Consts& kc, const float4* __restrict__ r,
		bool valid, const Tgt& g, float2 (&acc)[NC][kSymH], float (&js)[NC])
	{
		constexpr bool kFinite = FiniteAtZero<R>::value;
		const RegConsts& rc = kc.rc;
		float4 sp = r[0], sv = r[1];
		if (!FULL && !valid) {
			sp = make_float4(0.f, 0.f, 0.f, 0.f);
			sv = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		const float2 sx = bc2(sp.x), sy = bc2(sp.y), sz = bc2(sp.z);
		const float2 wx = bc2(sv.x), wy = bc2(sv.y), wz = bc2(sv.z);
		const float2 nwx = bc2(-sv.x), nwy = bc2(-sv.y), nwz = bc2(-sv.z);
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const float2 dx = __ffma2_rn(sx, bc2(-1.f), g.tx[h]);
			const float2 dy = __ffma2_rn(sy, bc2(-1.f), g.ty[h]);
			const float2 dz = __ffma2_rn(sz, bc2(-1.f), g.tz[h]);
			const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
			float2 G, K;
			if (DV) {
				RegP3D2<R>::gk2(r2, rc, G, K);
				G.x = r2.x > 0.f ? G.x : 0.f;
				G.y = r2.y > 0.f ? G.y : 0.f;
				if (!kFinite) {
					K.x = r2.x > 0.f ? K.x : 0.f;
					K.y = r2.y > 0.f ? K.y : 0.f;
				}
			} else {
				G = RegP3D2<R>::g2(r2, rc);
				if (!kFinite) {
					G.x = r2.x > 0.f ? G.x : 0.f;
					G.y = r2.y > 0.f ? G.y : 0.f;
				}
			}
			if (!FULL && !valid) {
				G = make_float2(0.f, 0.f);
				K = make_float2(0.f, 0.f);
			}
			if (VEL) {
				// e = G d, then t: e x alpha_s and s: alpha_t x e, the cross
				// products' terms added one by one (no separate cross product
				// per side: 1,859 -> 2,163 G/s for the velocity alone, 968 ->
				// 1,068 fused, 1M cube; FP64 error 2.9e-7 -> 4.0e-7)
				const float2 ex = __fmul2_rn(G, dx), ey = __fmul2_rn(G, dy), ez = __fmul2_rn(G, dz);
				acc[0][h] = __ffma2_rn(ey, wz, __ffma2_rn(ez, nwy, acc[0][h]));
				acc[1][h] = __ffma2_rn(ez, wx, __ffma2_rn(ex, nwz, acc[1][h]));
				acc[2][h] = __ffma2_rn(ex, wy, __ffma2_rn(ey, nwx, acc[2][h]));
				if (SYM) {
					js[0] = fmaf(g.ay[h].x, ez.x, fmaf(g.ay[h].y, ez.y,
						fmaf(g.naz[h].x, ey.x, fmaf(g.naz[h].y, ey.y, js[0]))));
					js[1] = fmaf(g.az[h].x, ex.x, fmaf(g.az[h].y, ex.y,
						fmaf(g.nax[h].x, ez.x, fmaf(g.nax[h].y, ez.y, js[1]))));
					js[2] = fmaf(g.ax[h].x, ey.x, fmaf(g.ax[h].y, ey.y,
						fmaf(g.nay[h].x, ex.x, fmaf(g.nay[h].y, ex.y, js[2]))));
				}
			}
			if (DV) {
				constexpr int o = VEL ? 3 : 0;
				// co = alpha_t x alpha_s (reference rounding)
				float2 ox, oy, oz;
				cross_ref2(g.ax[h], g.ay[h], g.az[h], wx, wy, wz, nwx, nwy, nwz, ox, oy, oz);
				const float2 pd = __ffma2_rn(dz, oz, __ffma2_rn(dy, oy, __fmul2_rn(dx, ox)));
				const float2 kk = __fmul2_rn(K, pd);
				acc[o + 0][h] = __ffma2_rn(G, ox, acc[o + 0][h]);
				acc[o + 1][h] = __ffma2_rn(G, oy, acc[o + 1][h]);
				acc[o + 2][h] = __ffma2_rn(G, oz, acc[o + 2][h]);
				acc[o + 3][h] = __ffma2_rn(kk, dx, acc[o + 3][h]);
				acc[o + 4][h] = __ffma2_rn(kk, dy, acc[o + 4][h]);
				acc[o + 5][h] = __ffma2_rn(kk, dz, acc[o + 5][h]);
				if (SYM) {
					js[o + 0] = fmaf(-G.x, ox.x, fmaf(-G.y, ox.y, js[o + 0]));
					js[o + 1] = fmaf(-G.x, oy.x, fmaf(-G.y, oy.y, js[o + 1]));
					js[o + 2] = fmaf(-G.x, oz.x, fmaf(-G.y, oz.y, js[o + 2]));
					js[o + 3] = fmaf(-kk.x, dx.x, fmaf(-kk.y, dx.y, js[o + 3]));
					js[o + 4] = fmaf(-kk.x, dy.x, fmaf(-kk.y, dy.y, js[o + 4]));
					js[o + 5] = fmaf(-kk.x, dz.x, fmaf(-kk.y, dz.y, js[o + 5]));
				}
			}
		}
	}

	__device__ __forceinline__ static void write(const Problem& p, const Consts& kc, int t,
		const double* s)
	{
		write_induce<VEL, DV>(p, kc, t, s);
	}

	// A diagonal item: the per-call CTA body over the block's ordered pairs.
	__device__ __forceinline__ static bool diagonal(const Problem& p, const Consts& kc,
		const SymArgs& a, int b, unsigned char* smem, unsigned* err, unsigned& tcount)
	{
		const int n = p.n_tgt;
		const int b0 = b * a.S;
		const int b1 = min(n, b0 + a.S);
		Problem q = p;
		q.n_tgt = b1;      // targets of this block only; loads clamp below b1
		for (int tb = b0; tb < b1; tb += kSymPass) {
			const bool ok = induce2_block<R, VEL, DV, kSymTPT, kSymNT, 2>(q, kc, tb, b0, b1 - b0,
				smem, err, tcount, [&](int t, const double* s) {
#pragma unroll
					for (int c = 0; c < NC; ++c) a.slots[(size_t(b) * NC + c) * n + t] = float(s[c]);
				});
			if (!ok) return false;
		}
		return true;
	}
};

// Viscous vorticity exchange (PSE, reference src/P3D.cpp:116-144): the
// per-pair difference alpha_s V_t - alpha_t V_s, formed as in the per-call
// kernels (p3d.cu), weighted by the shape of eta (its constant factor is in
// the FP64 output scale).
struct SymViscConsts { RegConsts rc; double scale; };

template <Reg R>
struct ViscSym {
	using Problem = P3DViscProblem;
	using Consts = SymViscConsts;
	static constexpr int NC = 3;
	// 100k ring, Winckelmans: unroll 16 -> 1,966, 8 -> 1,943, 4 -> 1,925,
	// 2 -> 1,821 G/s; Gaussian: 4 CTAs per SM, unroll 8 -> 2,232 (3 CTAs,
	// unroll 16: 2,155)
	static constexpr int kUnroll = R == Reg::Gaussian ? 8 : 16;
	static constexpr int kRec = 2, kTile = kP3DTile;
	static constexpr int kMinBlocks = R == Reg::Gaussian ? 4 : kP3DSymMinBlocks;
	static constexpr double kPlanFactor = 26.0;   // 100k ring: 2,027 against 1,999 with 16
	static constexpr bool kOwnDiagonal = false;
	struct Tgt {
		float2 ntx[kSymH], nty[kSymH], ntz[kSymH], tv[kSymH], nax[kSymH], nay[kSymH], naz[kSymH];
	};

	__device__ __forceinline__ static void load(const Problem& p, int tb, int tid, int lim,
		Tgt& g)
	{
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const int t0 = min(tb + (2 * h) * kSymNT + tid, lim - 1);
			const int t1 = min(tb + (2 * h + 1) * kSymNT + tid, lim - 1);
			const float4 q0 = p.tgt[2 * size_t(t0)], q1 = p.tgt[2 * size_t(t1)];
			const float4 v0 = p.tgt[2 * size_t(t0) + 1], v1 = p.tgt[2 * size_t(t1) + 1];
			g.ntx[h] = make_float2(-q0.x, -q1.x); g.nty[h] = make_float2(-q0.y, -q1.y);
			g.ntz[h] = make_float2(-q0.z, -q1.z); g.tv[h] = make_float2(q0.w, q1.w);
			g.nax[h] = make_float2(-v0.x, -v1.x); g.nay[h] = make_float2(-v0.y, -v1.y);
			g.naz[h] = make_float2(-v0.z, -v1.z);
		}
	}

	template <bool FULL, bool SYM>
	__device__ __forceinline__ static void step(const Consts& vc, const float4* __restrict__ r,
		bool valid, const Tgt& g, float2 (&acc)[NC][kSymH], float (&js)[NC])
	{
		float4 sp = r[0], sv = r[1];
		if (!FULL && !valid) {
			sp = make_float4(0.f, 0.f, 0.f, 0.f);
			sv = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		const float2 sx = bc2(sp.x), sy = bc2(sp.y), sz = bc2(sp.z), vs = bc2(sp.w);
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			// source - target, rounded once as in the per-call kernels
			const float2 dx = __fadd2_rn(sx, g.ntx[h]);
			const float2 dy = __fadd2_rn(sy, g.nty[h]);
			const float2 dz = __fadd2_rn(sz, g.ntz[h]);
			const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
			float2 e = RegEta2<R>::eta2(r2, vc.rc);
			e.x = r2.x > 0.f ? e.x : 0.f;
			e.y = r2.y > 0.f ? e.y : 0.f;
			if (!FULL && !valid) e = make_float2(0.f, 0.f);
			// alpha_s V_t - alpha_t V_s
			const float2 wx = __ffma2_rn(bc2(sv.x), g.tv[h], __fmul2_rn(g.nax[h], vs));
			const float2 wy = __ffma2_rn(bc2(sv.y), g.tv[h], __fmul2_rn(g.nay[h], vs));
			const float2 wz = __ffma2_rn(bc2(sv.z), g.tv[h], __fmul2_rn(g.naz[h], vs));
			acc[0][h] = __ffma2_rn(e, wx, acc[0][h]);
			acc[1][h] = __ffma2_rn(e, wy, acc[1][h]);
			acc[2][h] = __ffma2_rn(e, wz, acc[2][h]);
			if (SYM) {
				js[0] = fmaf(-e.x, wx.x, fmaf(-e.y, wx.y, js[0]));
				js[1] = fmaf(-e.x, wy.x, fmaf(-e.y, wy.y, js[1]));
				js[2] = fmaf(-e.x, wz.x, fmaf(-e.y, wz.y, js[2]));
			}
		}
	}

	__device__ __forceinline__ static void write(const Problem& p, const Consts& vc, int t,
		const double* s)
	{
		float* o = p.out + 3 * size_t(t);
		o[0] = float(vc.scale * s[0]);
		o[1] = float(vc.scale * s[1]);
		o[2] = float(vc.scale * s[2]);
	}
};

// Vorticity field at the particles' own positions (reference
// src/P3D.cpp:298-322, the CPU path with its 5 sigma box): the pair's weight
// zeta(r) and its box test (on |d_x|, |d_y|, |d_z|, unchanged when d changes
// sign) serve both particles: t gets zeta alpha_s, s gets zeta alpha_t. The
// pair of a particle with itself counts once, as in the reference.
struct SymVortConsts { RegConsts rc; float cutoff; double scale; };

template <Reg R>
struct VortSym {
	using Problem = P3DVortProblem;
	using Consts = SymVortConsts;
	static constexpr int NC = 3;
	// 100k ring, G/s: 4 CTAs per SM (128 registers) 2,629 / 3,091 / 2,976
	// (Winckelmans / planetary / Gaussian), 3 CTAs 2,545 / 2,876 / 2,852
	static constexpr int kUnroll = 8;
	static constexpr double kFactor = ZetaShape2<R>::kFactor;   // in the output scale
	static constexpr int kRec = 2, kTile = kP3DTile, kMinBlocks = 4;
	static constexpr double kPlanFactor = 16.0;   // 100k ring: 2,680 against 2,625 with 26
	static constexpr bool kOwnDiagonal = false;
	struct Tgt {
		float2 ntx[kSymH], nty[kSymH], ntz[kSymH], ax[kSymH], ay[kSymH], az[kSymH];
	};

	__device__ __forceinline__ static void load(const Problem& p, int tb, int tid, int lim,
		Tgt& g)
	{
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			const int t0 = min(tb + (2 * h) * kSymNT + tid, lim - 1);
			const int t1 = min(tb + (2 * h + 1) * kSymNT + tid, lim - 1);
			const float4 q0 = p.tgt[2 * size_t(t0)], q1 = p.tgt[2 * size_t(t1)];
			const float4 v0 = p.tgt[2 * size_t(t0) + 1], v1 = p.tgt[2 * size_t(t1) + 1];
			g.ntx[h] = make_float2(-q0.x, -q1.x); g.nty[h] = make_float2(-q0.y, -q1.y);
			g.ntz[h] = make_float2(-q0.z, -q1.z);
			g.ax[h] = make_float2(v0.x, v1.x); g.ay[h] = make_float2(v0.y, v1.y);
			g.az[h] = make_float2(v0.z, v1.z);
		}
	}

	template <bool FULL, bool SYM>
	__device__ __forceinline__ static void step(const Consts& kc, const float4* __restrict__ r,
		bool valid, const Tgt& g, float2 (&acc)[NC][kSymH], float (&js)[NC])
	{
		float4 sp = r[0], sv = r[1];
		if (!FULL && !valid) {
			sp = make_float4(0.f, 0.f, 0.f, 0.f);
			sv = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		const float2 sx = bc2(sp.x), sy = bc2(sp.y), sz = bc2(sp.z);
#pragma unroll
		for (int h = 0; h < kSymH; ++h) {
			// source - target, rounded once as in the per-call kernels
			const float2 dx = __fadd2_rn(sx, g.ntx[h]);
			const float2 dy = __fadd2_rn(sy, g.nty[h]);
			const float2 dz = __fadd2_rn(sz, g.ntz[h]);
			const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
			float2 z = ZetaShape2<R>::z(r2, kc.rc);
			const bool in0 = max3_nan(fabsf(dx.x), fabsf(dy.x), fabsf(dz.x)) < kc.cutoff;
			const bool in1 = max3_nan(fabsf(dx.y), fabsf(dy.y), fabsf(dz.y)) < kc.cutoff;
			z.x = in0 ? z.x : 0.f;
			z.y = in1 ? z.y : 0.f;
			if (!FULL && !valid) z = make_float2(0.f, 0.f);
			acc[0][h] = __ffma2_rn(z, bc2(sv.x), acc[0][h]);
			acc[1][h] = __ffma2_rn(z, bc2(sv.y), acc[1][h]);
			acc[2][h] = __ffma2_rn(z, bc2(sv.z), acc[2][h]);
			if (SYM) {
				js[0] = fmaf(z.x, g.ax[h].x, fmaf(z.y, g.ax[h].y, js[0]));
				js[1] = fmaf(z.x, g.ay[h].x, fmaf(z.y, g.ay[h].y, js[1]));
				js[2] = fmaf(z.x, g.az[h].x, fmaf(z.y, g.az[h].y, js[2]));
			}
		}
	}

	__device__ __forceinline__ static void write(const Problem& p, const Consts& kc, int t,
		const double* s)
	{
		float* o = p.out + 3 * size_t(t);
		o[0] = float(kc.scale * s[0]);
		o[1] = float(kc.scale * s[1]);
		o[2] = float(kc.scale * s[2]);
	}
};

// ---- many problems (the batched form) -----------------------------------------
// Persistent CTAs claim (problem, bi, bj) items; each item runs exactly as in
// the single-problem kernel, on its problem's blocks and slots.
template <class Op>
__global__ void __launch_bounds__(kSymNT, Op::kMinBlocks)
sym_batch_kernel(const SymBatchProblem* __restrict__ probs, int n_probs,
	const int4* __restrict__ items, int n_items, unsigned* next, unsigned* err)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__shared__ SymBatchProblem sp;
	__shared__ int item_s;
	if (blockDim.x != kSymNT) {
		if (threadIdx.x == 0) atomicOr(err, kErrBadLaunch);
		return;
	}
	if (!SymStream<Op>::init(smem, err)) return;
	unsigned tcount = 0;
	for (;;) {
		if (threadIdx.x == 0) item_s = int(atomicAdd(next, 1u));
		__syncthreads();
		const int it = item_s;
		__syncthreads();
		if (it >= n_items) return;
		const int4 w = items[it];
		if (w.x < 0 || w.x >= n_probs) {
			if (threadIdx.x == 0) atomicOr(err, kErrBadWork);
			continue;
		}
		// every thread finished its reads of the previous problem before
		// the two barriers above
		if (threadIdx.x == 0) sp = probs[w.x];
		__syncthreads();
		const int bi = w.y, bj = w.z;
		if (bi < 0 || bj < bi || bj >= sp.nb || bi * sp.S >= sp.p.n_tgt) {
			if (threadIdx.x == 0) atomicOr(err, kErrBadWork);
			continue;
		}
		SymArgs a;
		a.S = sp.S;
		a.nb = sp.nb;
		a.slots = sp.slots;
		const bool ok = bi == bj ? sym_diagonal<Op>(sp.p, sp.kc, a, bi, smem, err, tcount)
		                         : sym_item<Op, true>(sp.p, sp.kc, a, bi, bj, smem, err, tcount);
		if (!ok) return;
	}
}

// Every particle of every problem: its nb slot partials in block order
// (FP64), then the output transforms.
template <class Op>
__global__ void sym_batch_finalize(const SymBatchProblem* __restrict__ probs,
	const int* __restrict__ prefix, int n_probs, int total)
{
	constexpr int NC = Op::NC;
	const int g = blockIdx.x * blockDim.x + threadIdx.x;
	if (g >= total) return;
	int lo = 0, hi = n_probs - 1;      // the problem with prefix[i] <= g
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (prefix[mid] <= g) lo = mid;
		else hi = mid - 1;
	}
	const SymBatchProblem& q = probs[lo];
	const int n = q.p.n_tgt;
	const int t = g - prefix[lo];
	if (t < 0 || t >= n) return;
	double s[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) s[c] = 0.0;
	for (int b = 0; b < q.nb; ++b)
#pragma unroll
		for (int c = 0; c < NC; ++c) s[c] += double(q.slots[(size_t(b) * NC + c) * n + t]);
	Op::write(q.p, q.kc, t, s);
}

template <class Op>
int sym_batch_occupancy() {
	static const int occ = resident_ctas(sym_batch_kernel<Op>, kSymNT, sym_smem_bytes<Op>());
	return occ;
}

template <class F>
auto with_reg_vort(int reg, F&& f) {
	switch (reg) {
	case 1: return f(static_cast<VortSym<Reg::Winckelmans>*>(nullptr));
	case 2: return f(static_cast<VortSym<Reg::Planetary>*>(nullptr));
	default: return f(static_cast<VortSym<Reg::Gaussian>*>(nullptr));
	}
}

template <class F>
auto with_reg_ops_sym(int reg, unsigned ops, F&& f) {
	auto by_ops = [&](auto rt) {
		constexpr Reg R = decltype(rt)::value;
		if (ops == kOpVel) return f(static_cast<InduceSym<R, true, false>*>(nullptr));
		if (ops == kOpDvort) return f(static_cast<InduceSym<R, false, true>*>(nullptr));
		return f(static_cast<InduceSym<R, true, true>*>(nullptr));
	};
	switch (reg) {
	case 0: return by_ops(std::integral_constant<Reg, Reg::Singular>{});
	case 1: return by_ops(std::integral_constant<Reg, Reg::Winckelmans>{});
	case 2: return by_ops(std::integral_constant<Reg, Reg::Planetary>{});
	default: return by_ops(std::integral_constant<Reg, Reg::Gaussian>{});
	}
}

bool self_shape(const float4* src, int n_src, const float4* tgt, int tstride, int n_tgt) {
	return tgt == src && tstride == 2 && n_tgt == n_src && sym_size_ok(n_tgt);
}

}  // namespace

// Measured on a GB300 against the ordered-pair kernel (G interactions/s):
// fused 1,079 against 866 (1M cube), stretching alone 1,523 against 1,010 and
// velocity alone 2,110 against 1,722 (100,000-particle ring).
bool p3d_self_form_applies(int reg, unsigned ops, const P3DInduceProblem& p) {
	(void)reg;
	(void)ops;
	return self_shape(p.src, p.n_src, p.tgt, p.tstride, p.n_tgt);
}

size_t p3d_self_ws_bytes(int reg, unsigned ops, int n, int num_sms, size_t ws_cap) {
	return with_reg_ops_sym(reg, ops, [&](auto* op) {
		using Op = std::remove_pointer_t<decltype(op)>;
		return sym_ws_bytes<Op>(n, num_sms, ws_cap);
	});
}

cudaError_t p3d_self(int reg, unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env) {
	return with_reg_ops_sym(reg, ops, [&](auto* op) {
		using Op = std::remove_pointer_t<decltype(op)>;
		return sym_launch<Op>(p, make_induce_consts(reg, p.sigma), env);
	});
}

bool p3d_visc_self_form_applies(int reg, const P3DViscProblem& p) {
	return (reg == int(Reg::Winckelmans) || reg == int(Reg::Gaussian)) &&
		self_shape(p.src, p.n_src, p.tgt, p.tstride, p.n_tgt);
}

size_t p3d_visc_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap) {
	return reg == int(Reg::Winckelmans) ? sym_ws_bytes<ViscSym<Reg::Winckelmans>>(n, num_sms, ws_cap)
	                                    : sym_ws_bytes<ViscSym<Reg::Gaussian>>(n, num_sms, ws_cap);
}

cudaError_t p3d_visc_self(int reg, const P3DViscProblem& p, const LaunchEnv& env) {
	SymViscConsts vc;
	vc.rc = make_reg_consts_host(p.sigma);
	const double base = 2.0 * double(p.nu) / (double(p.sigma) * double(p.sigma));
	if (reg == int(Reg::Winckelmans)) {
		vc.scale = base * 52.5;
		return sym_launch<ViscSym<Reg::Winckelmans>>(p, vc, env);
	}
	if (reg == int(Reg::Gaussian)) {
		vc.scale = base * double(kSqrt2OverPi);
		return sym_launch<ViscSym<Reg::Gaussian>>(p, vc, env);
	}
	return cudaErrorInvalidValue;
}

int p3d_sym_batch_occupancy(int reg, unsigned ops) {
	return with_reg_ops_sym(reg, ops, [&](auto* op) {
		using Op = std::remove_pointer_t<decltype(op)>;
		return sym_batch_occupancy<Op>();
	});
}

cudaError_t p3d_sym_batch_enqueue(int reg, unsigned ops, const SymBatchProblem* probs,
	int n_probs, const int4* items, int n_items, const int* prefix, int total, unsigned* next,
	unsigned* err, int grid, cudaStream_t s)
{
	if (n_probs <= 0 || n_items <= 0) return cudaSuccess;
	return with_reg_ops_sym(reg, ops, [&](auto* op) {
		using Op = std::remove_pointer_t<decltype(op)>;
		sym_batch_kernel<Op><<<std::max(grid, 1), kSymNT, sym_smem_bytes<Op>(), s>>>(
			probs, n_probs, items, n_items, next, err);
		count_launch();
		sym_batch_finalize<Op><<<(total + 255) / 256, 256, 0, s>>>(probs, prefix, n_probs, total);
		count_launch();
		return cudaGetLastError();
	});
}

bool p3d_vort_self_form_applies(int reg, const P3DVortProblem& p) {
	return reg >= 1 && reg <= 3 && self_shape(p.src, p.n_src, p.tgt, p.tstride, p.n_tgt);
}

size_t p3d_vort_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap) {
	return with_reg_vort(reg, [&](auto* op) {
		using Op = std::remove_pointer_t<decltype(op)>;
		return sym_ws_bytes<Op>(n, num_sms, ws_cap);
	});
}

cudaError_t p3d_vort_self(int reg, const P3DVortProblem& p, const LaunchEnv& env) {
	if (reg < 1 || reg > 3) return cudaErrorInvalidValue;
	return with_reg_vort(reg, [&](auto* op) {
		using Op = std::remove_pointer_t<decltype(op)>;
		const double s = p.sigma;
		SymVortConsts kc;
		kc.rc = make_reg_consts_host(p.sigma);
		kc.cutoff = 5.f * p.sigma;
		kc.scale = Op::kFactor / (4.0 * 3.14159265358979323846 * s * s * s);
		return sym_launch<Op>(p, kc, env);
	});
}

}  // namespace cvtx
