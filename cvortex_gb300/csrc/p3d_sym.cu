// p3d_sym.cu -- P3D interactions of a particle set on itself, each unordered
// pair evaluated once: vortex stretching (with or without the velocity) and
// the viscous vorticity exchange.
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
// Work decomposition (deterministic, no floating-point atomics):
// * The particles are cut into nb blocks of S (a multiple of the 512-target
//   pass of a CTA; the last block may be shorter). A work item is a block
//   pair (bi, bj), bi <= bj; a persistent grid claims items through an atomic
//   counter, largest first.
// * Item (bi, bj), bi < bj: for each pass of 512 particles of block bi (held
//   in registers, two per f32x2 lane pair), the records of block bj stream
//   through shared memory in 256-record tiles (bulk copies). Within a warp
//   the 32 records of a group are visited in a rotation: at step k lane l
//   pairs its four particles with record (l + k) mod 32, whose running sums
//   travel with it from lane to lane by shuffles and are back at their home
//   lane after 32 steps. The four warps' sums per record are added in warp
//   order in shared memory and added into the workspace slot (bi, record).
//   The bi particles' own sums are folded per tile into compensated
//   (hi, lo) pairs and written to slot (bj, particle) after the pass.
// * Item (b, b): every ordered pair of the block, into slot (b, particle):
//   the per-call CTA body (induce2_block) for the induced velocity and
//   stretching, the same rotation with the record side left out for the
//   viscous exchange.
// * Every particle thus has exactly nb slot partials (one per partner
//   block); a finalize kernel adds them in block order in FP64 and applies
//   the output transforms. The result does not depend on scheduling.
//
// Coincident distinct particles contribute nothing to each other, as in the
// reference; every wait on a tile is bounded (tile_stream.cuh).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <type_traits>

#include "nbody.h"
#include "p3d_induce.cuh"
#include "plan.cuh"

namespace cvtx {

// Regularisation constants for one regularisation distance (p3d.cu).
RegConsts make_reg_consts_host(float sigma);

namespace {

constexpr int kSymNT = 128;                    // threads per CTA
constexpr int kSymTPT = 4;                     // particles per thread and pass
constexpr int kSymH = kSymTPT / 2;             // f32x2 lane pairs per thread
constexpr int kSymPass = kSymNT * kSymTPT;     // particles of block bi per pass
constexpr int kSymWarps = kSymNT / 32;
// Resident CTAs per SM the registers are sized for (167 registers for the
// fused pair). Sizing for two (217 registers) measured 5-7 % slower.
constexpr int kSymMinBlocks = 3;

// ---- pair operations -------------------------------------------------------
// An operation supplies: NC sums per particle; the per-lane particle data
// (Tgt: four particles as two f32x2 lane pairs) and its loader (indices
// clamped below `lim`); step<FULL, SYM>, one lane's particles against one
// record, adding to the particles' packed sums `acc` and (SYM) to the
// record's running sums `js`; write, the output of a particle from its FP64
// sums; kUnroll, the rotation steps unrolled (timed on a GB300 per op; two
// particles per thread instead of four measured 5-9 % slower).
// FULL = false zeroes the pair for a lane whose record lies past the
// end of the block (`valid` false).

// Induced velocity and/or stretching (reference src/P3D.cpp:51-114).
template <Reg R, bool VEL, bool DV>
struct InduceSym {
	using Problem = P3DInduceProblem;
	using Consts = InduceConsts;
	static constexpr int NC = InduceNC<VEL, DV>::value;
	// fused, 1M cube: 4 -> 967, 8 -> 947, 2 -> 937 G/s; one output alone: 8
	static constexpr int kUnroll = (VEL && DV) ? 4 : 8;
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
	__device__ __forceinline__ static void step(const Consts& kc, float4 sp, float4 sv,
		bool valid, const Tgt& g, float2 (&acc)[NC][kSymH], float (&js)[NC])
	{
		constexpr bool kFinite = FiniteAtZero<R>::value;
		const RegConsts& rc = kc.rc;
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
				// t: G d x alpha_s; s: -G d x alpha_t
				const float2 cx = __ffma2_rn(dy, wz, __fmul2_rn(dz, nwy));
				const float2 cy = __ffma2_rn(dz, wx, __fmul2_rn(dx, nwz));
				const float2 cz = __ffma2_rn(dx, wy, __fmul2_rn(dy, nwx));
				acc[0][h] = __ffma2_rn(G, cx, acc[0][h]);
				acc[1][h] = __ffma2_rn(G, cy, acc[1][h]);
				acc[2][h] = __ffma2_rn(G, cz, acc[2][h]);
				if (SYM) {
					const float2 qx = __ffma2_rn(dy, g.az[h], __fmul2_rn(dz, g.nay[h]));
					const float2 qy = __ffma2_rn(dz, g.ax[h], __fmul2_rn(dx, g.naz[h]));
					const float2 qz = __ffma2_rn(dx, g.ay[h], __fmul2_rn(dy, g.nax[h]));
					js[0] = fmaf(-G.x, qx.x, fmaf(-G.y, qx.y, js[0]));
					js[1] = fmaf(-G.x, qy.x, fmaf(-G.y, qy.y, js[1]));
					js[2] = fmaf(-G.x, qz.x, fmaf(-G.y, qz.y, js[2]));
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
	// 100k ring: 16 -> 1,966, 8 -> 1,943, 4 -> 1,925, 2 -> 1,821 G/s
	static constexpr int kUnroll = 16;
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
	__device__ __forceinline__ static void step(const Consts& vc, float4 sp, float4 sv,
		bool valid, const Tgt& g, float2 (&acc)[NC][kSymH], float (&js)[NC])
	{
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

// ---- the rotation ------------------------------------------------------------
template <int NC>
constexpr size_t sym_smem_bytes() {
	// tile stages, (hi, lo) per pass particle and sum, and two buffers of
	// per-warp record sums [2][warps][NC][32]
	return P3DStream::kSmemBytes + size_t(2) * NC * kSymPass * sizeof(float) +
		size_t(2) * kSymWarps * NC * 32 * sizeof(float);
}

// Fire-and-forget add to global memory (no value returned, so the thread
// does not wait for it).
__device__ __forceinline__ void red_add_f32(float* p, float v) {
	asm volatile("red.global.add.f32 [%0], %1;" :: "l"(p), "f"(v) : "memory");
}

// One 32-record group: 32 rotation steps; with SYM the group records' sums
// come back at their home lanes in js. (Passing the records' data along
// with their sums by shuffles, instead of reading them from shared memory at
// every step, measured no faster on a GB300.)
template <class Op, bool FULL, bool SYM>
__device__ __forceinline__ void sym_group(const typename Op::Consts& kc,
	const float4* __restrict__ grp, int gcnt, int lane, const typename Op::Tgt& g,
	float2 (&acc)[Op::NC][kSymH], float (&js)[Op::NC])
{
	const int from = (lane + 1) & 31;
#pragma unroll Op::kUnroll
	for (int k = 0; k < 32; ++k) {
		const int jl = (lane + k) & 31;
		const float4 sp = grp[2 * jl];
		const float4 sv = grp[2 * jl + 1];
		Op::template step<FULL, SYM>(kc, sp, sv, jl < gcnt, g, acc, js);
		if (SYM) {
#pragma unroll
			for (int c = 0; c < Op::NC; ++c) js[c] = __shfl_sync(0xffffffffu, js[c], from);
		}
	}
}

struct SymArgs {
	int S;            // block length (multiple of kSymPass)
	int nb;           // blocks
	float* slots;     // [nb][NC][n] partial sums
};

// Item (bi, bj): all passes of block bi against block bj. SYM (bi < bj)
// also adds the bj records' sums into their slots (bi, record); without it
// (a diagonal item) only the bi particles' sums are formed. Returns false if
// a tile wait timed out.
template <class Op, bool SYM>
__device__ __forceinline__ bool sym_item(const typename Op::Problem& p,
	const typename Op::Consts& kc, const SymArgs& a, int bi, int bj, unsigned char* smem,
	unsigned* err, unsigned& tcount)
{
	constexpr int NC = Op::NC;
	const int n = p.n_tgt;
	float* hi = reinterpret_cast<float*>(smem + P3DStream::kSmemBytes);
	float* lo = hi + NC * kSymPass;
	float* jbuf = lo + NC * kSymPass;            // [2][warps][NC][32]
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int i0 = bi * a.S;
	const int i1 = min(n, i0 + a.S);              // whole passes when bi < bj
	const int j0 = bj * a.S;
	const int nj = min(n, j0 + a.S) - j0;
	int par = 0;
	for (int tb = i0; tb < i1; tb += kSymPass) {
		typename Op::Tgt g;
		Op::load(p, tb, tid, i1, g);
#pragma unroll
		for (int i = 0; i < NC * kSymTPT; ++i) { hi[i * kSymNT + tid] = 0.f; lo[i * kSymNT + tid] = 0.f; }
		int toff = 0;   // first record of the current tile within block bj

		auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
			float2 acc[NC][kSymH];
#pragma unroll
			for (int c = 0; c < NC; ++c)
#pragma unroll
				for (int h = 0; h < kSymH; ++h) acc[c][h] = make_float2(0.f, 0.f);
			const int ng = (cnt + 31) >> 5;
			for (int gi = 0; gi < ng; ++gi) {
				const int gcnt = min(32, cnt - 32 * gi);
				const float4* grp = st + 2 * 32 * gi;
				float js[NC];
#pragma unroll
				for (int c = 0; c < NC; ++c) js[c] = 0.f;
				if (gcnt == 32) sym_group<Op, true, SYM>(kc, grp, gcnt, lane, g, acc, js);
				else sym_group<Op, false, SYM>(kc, grp, gcnt, lane, g, acc, js);
				if (SYM) {
					// the group's record sums are back at their home lanes
					float* wb = jbuf + ((par * kSymWarps + warp) * NC) * 32;
#pragma unroll
					for (int c = 0; c < NC; ++c) wb[c * 32 + lane] = js[c];
					__syncthreads();
					// warp-ordered sum per record, added to its slot (zeroed
					// before the launch). A slot element is only ever added to
					// by this thread of this CTA, in pass order, so the sum is
					// deterministic; the reduction does not wait for the memory.
					const float* rb = jbuf + (par * kSymWarps * NC) * 32;
					for (int v = tid; v < NC * 32; v += kSymNT) {
						const int c = v >> 5, l = v & 31;
						if (l >= gcnt) continue;
						float s = rb[v];
#pragma unroll
						for (int w = 1; w < kSymWarps; ++w) s += rb[w * NC * 32 + v];
						red_add_f32(a.slots + (size_t(bi) * NC + c) * n +
							(j0 + toff + 32 * gi + l), s);
					}
					par ^= 1;
				}
			}
#pragma unroll
			for (int c = 0; c < NC; ++c) {
#pragma unroll
				for (int h = 0; h < kSymH; ++h)
#pragma unroll
					for (int e = 0; e < 2; ++e) {
						const int i = (c * kSymTPT + 2 * h + e) * kSymNT + tid;
						float hh = hi[i], ll = lo[i];
						fold_twosum(hh, ll, e == 0 ? acc[c][h].x : acc[c][h].y);
						hi[i] = hh; lo[i] = ll;
					}
			}
			toff += cnt;
		};
		if (!P3DStream::run_continue(smem, p.src, j0, nj, err, tcount, tile_fn)) return false;
#pragma unroll
		for (int k = 0; k < kSymTPT; ++k) {
			const int t = tb + k * kSymNT + tid;
			if (t >= i1) continue;
#pragma unroll
			for (int c = 0; c < NC; ++c) {
				const int i = (c * kSymTPT + k) * kSymNT + tid;
				a.slots[(size_t(bj) * NC + c) * n + t] = float(double(hi[i]) + double(lo[i]));
			}
		}
	}
	return true;
}

// The diagonal item (b, b) of the induced velocity / stretching: the per-call
// CTA body over the block's ordered pairs.
template <Reg R, bool VEL, bool DV>
__device__ __forceinline__ bool sym_diagonal(const P3DInduceProblem& p, const InduceConsts& kc,
	const SymArgs& a, int b, unsigned char* smem, unsigned* err, unsigned& tcount,
	InduceSym<R, VEL, DV>*)
{
	constexpr int NC = InduceNC<VEL, DV>::value;
	const int n = p.n_tgt;
	const int b0 = b * a.S;
	const int b1 = min(n, b0 + a.S);
	P3DInduceProblem q = p;
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

template <Reg R>
__device__ __forceinline__ bool sym_diagonal(const P3DViscProblem& p, const SymViscConsts& vc,
	const SymArgs& a, int b, unsigned char* smem, unsigned* err, unsigned& tcount, ViscSym<R>*)
{
	return sym_item<ViscSym<R>, false>(p, vc, a, b, b, smem, err, tcount);
}

// Item `it` of nb blocks, largest first: the full off-diagonal pairs column
// by column (bj = 1 .. nb-2, bi < bj; items running at the same time share
// their bj block in L2), then the pairs with the short last block, then the
// diagonal blocks (about 2/3 of an off-diagonal pair's time).
__device__ __forceinline__ int2 sym_item_at(int it, int nb) {
	const long long a = (long long)(nb - 1) * (nb - 2) / 2;
	if (it < a) {
		long long j = (long long)((1.0 + sqrt(1.0 + 8.0 * double(it))) * 0.5);
		while (j * (j - 1) / 2 > it) --j;
		while ((j + 1) * j / 2 <= it) ++j;
		return make_int2(int(it - j * (j - 1) / 2), int(j));
	}
	if (it < a + nb - 1) return make_int2(int(it - a), nb - 1);
	const int b = int(it - a - (nb - 1));
	return make_int2(b, b);
}

template <class Op>
__global__ void __launch_bounds__(kSymNT, kSymMinBlocks)
p3d_sym_kernel(const typename Op::Problem p, const typename Op::Consts kc, const SymArgs a,
	int n_items, unsigned* next, unsigned* err)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__shared__ int item_s;
	if (blockDim.x != kSymNT) {
		if (threadIdx.x == 0) atomicOr(err, kErrBadLaunch);
		return;
	}
	if (!P3DStream::init(smem, err)) return;
	unsigned tcount = 0;
	const int n = p.n_tgt;
	for (;;) {
		if (threadIdx.x == 0) item_s = int(atomicAdd(next, 1u));
		__syncthreads();
		const int it = item_s;
		__syncthreads();
		if (it >= n_items) return;
		const int2 w = sym_item_at(it, a.nb);
		const int bi = w.x, bj = w.y;
		if (bi < 0 || bj < bi || bj >= a.nb || bi * a.S >= n) {
			if (threadIdx.x == 0) atomicOr(err, kErrBadWork);
			continue;
		}
		const bool ok = bi == bj
			? sym_diagonal(p, kc, a, bi, smem, err, tcount, static_cast<Op*>(nullptr))
			: sym_item<Op, true>(p, kc, a, bi, bj, smem, err, tcount);
		if (!ok) return;
	}
}

// Sum of every particle's nb slot partials in block order (FP64), then the
// output transforms.
template <class Op>
__global__ void p3d_sym_finalize(const typename Op::Problem p, const typename Op::Consts kc,
	const float* __restrict__ slots, int nb)
{
	constexpr int NC = Op::NC;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	const int n = p.n_tgt;
	if (t >= n) return;
	double s[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) s[c] = 0.0;
	for (int b = 0; b < nb; ++b)
#pragma unroll
		for (int c = 0; c < NC; ++c) s[c] += double(slots[(size_t(b) * NC + c) * n + t]);
	Op::write(p, kc, t, s);
}

template <class Op>
int sym_occupancy() {
	static const int occ = resident_ctas(p3d_sym_kernel<Op>, kSymNT, sym_smem_bytes<Op::NC>());
	return occ;
}

// Block plan: about eight items per resident CTA (so that the last items
// leave little of the GPU idle), blocks a multiple of the 512-particle pass,
// and a workspace within `ws_cap` bytes (fewer, longer blocks otherwise).
struct SymPlan {
	int S = 0, nb = 0, n_items = 0;
	size_t slots_bytes = 0, counter_off = 0, ws_bytes = 0;
};

SymPlan sym_plan(int n, int nc, int capacity, size_t ws_cap) {
	SymPlan pl;
	int nb = int(std::ceil(std::sqrt(16.0 * capacity)));
	for (;; nb = nb * 7 / 8) {
		nb = std::max(nb, 2);
		int S = (n + nb - 1) / nb;
		S = ((S + kSymPass - 1) / kSymPass) * kSymPass;
		const int nbr = (n + S - 1) / S;
		pl.S = S;
		pl.nb = nbr;
		pl.n_items = nbr * (nbr + 1) / 2;
		pl.slots_bytes = size_t(nbr) * nc * size_t(n) * sizeof(float);
		pl.slots_bytes = (pl.slots_bytes + 255) & ~size_t(255);
		pl.counter_off = pl.slots_bytes;
		pl.ws_bytes = pl.counter_off + 256;
		if (pl.ws_bytes <= ws_cap || nb == 2) break;
	}
	return pl;
}

// Largest workspace the self-interaction form asks of its caller (the slots
// grow as blocks x particles: 1M particles, fused: 3.1 GB; 4M: 14 GB).
constexpr size_t kSymWsCap = size_t(16) << 30;

// The workspace of the form, or SIZE_MAX where the cap leaves fewer than two
// items per resident CTA (blocks so long that the GPU would idle; the
// ordered-pair kernels then serve the call).
template <class Op>
size_t sym_ws_bytes(int n, int num_sms, size_t ws_cap) {
	const int capacity = num_sms * sym_occupancy<Op>();
	const SymPlan pl = sym_plan(n, Op::NC, capacity, ws_cap ? ws_cap : kSymWsCap);
	return pl.n_items < 2 * capacity ? SIZE_MAX : pl.ws_bytes;
}

template <class Op>
cudaError_t sym_launch(const typename Op::Problem& p, const typename Op::Consts& kc,
	const LaunchEnv& env)
{
	const int occ = sym_occupancy<Op>();
	const SymPlan pl = sym_plan(p.n_tgt, Op::NC, env.num_sms * occ,
		env.cap_to_ws ? env.ws_bytes : std::min(env.ws_bytes, kSymWsCap));
	if (pl.ws_bytes > env.ws_bytes || !env.ws) return cudaErrorInvalidValue;
	unsigned char* ws = static_cast<unsigned char*>(env.ws);
	unsigned* d_next = reinterpret_cast<unsigned*>(ws + pl.counter_off);
	// the slots and the item counter start at zero
	const cudaError_t e = cudaMemsetAsync(ws, 0, pl.ws_bytes, env.stream);
	if (e != cudaSuccess) return e;
	SymArgs a;
	a.S = pl.S;
	a.nb = pl.nb;
	a.slots = reinterpret_cast<float*>(ws);
	const int grid = std::max(1, std::min(pl.n_items, env.num_sms * occ));
	p3d_sym_kernel<Op><<<grid, kSymNT, sym_smem_bytes<Op::NC>(), env.stream>>>(
		p, kc, a, pl.n_items, d_next, env.err);
	count_launch();
	p3d_sym_finalize<Op><<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(p, kc, a.slots, pl.nb);
	count_launch();
	return cudaGetLastError();
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

int sym_min_particles() {
	static const int min_n = [] {
		const char* e = std::getenv("CVTX_GB300_SYM_MIN");
		return (e && *e) ? std::atoi(e) : 32768;
	}();
	return min_n;
}

bool self_shape(const float4* src, int n_src, const float4* tgt, int tstride, int n_tgt) {
	const int min_n = sym_min_particles();
	return min_n > 0 && tgt == src && tstride == 2 && n_tgt == n_src && n_tgt >= min_n &&
		n_tgt >= 2 * kSymPass;
}

}  // namespace

// Measured on a GB300 against the ordered-pair kernel (G interactions/s):
// fused 967 against 866 (1M cube), stretching alone 1,464 against 1,010 and
// velocity alone 1,770 against 1,698 (100,000-particle ring).
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

}  // namespace cvtx
