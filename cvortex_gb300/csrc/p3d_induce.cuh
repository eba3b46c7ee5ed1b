// p3d_induce.cuh -- the P3D velocity / vortex-stretching CTA body shared by
// the per-call kernels (p3d.cu) and the batched persistent kernel (batch.cu).
//
// Per pair (t, s), d = x_t - x_s, the sums per target (registers, FP32,
// reset every tile) are
//   VEL: u += G c,  c  = d x alpha_s
//   DV : A += G co, co = alpha_t x alpha_s
//        B += K (d.co) d
// with the reference's own per-pair terms (src/P3D.cpp:51-72, 86-114). The
// stretching cross product co is rounded as the reference rounds it (two
// products and a difference, no fused multiply-add), so that it is the
// reference's term bit for bit: its rounding is what decides the result
// both where the vorticity of a pair is nearly parallel (co small against
// |alpha_t||alpha_s|) and where a target's vorticity dwarfs its sources'
// (a factored or centred sum over the sources would cancel there).
// Across tiles the sums are compensated (hi, lo) pairs in shared memory.
// Final outputs: vel = S_vel u, dvort = S_dv (A - K_scale B).
#pragma once
#include "nbody.h"
#include "regfuncs.cuh"
#include "tile_stream.cuh"

namespace cvtx {

constexpr int kP3DTile = 256;
template <int TILE> using P3DStreamT = TileStream<2, TILE, 2>;
using P3DStream = P3DStreamT<kP3DTile>;

template <Reg R> struct FiniteAtZero { static constexpr bool value = true; };
template <> struct FiniteAtZero<Reg::Singular> { static constexpr bool value = false; };

// The shape of zeta for two pairs at a time (f32x2). zeta's constant factor
// (7.5 Winckelmans, 3 planetary, sqrt(2/pi) Gaussian) is left to the FP64
// output scale, so each pair evaluates only the shape of zeta.
template <Reg R> struct ZetaShape2;
template <> struct ZetaShape2<Reg::Winckelmans> {
	static constexpr double kFactor = 7.5;
	__device__ __forceinline__ static float2 z(float2 r2, const RegConsts& c) {
		const float2 q = __ffma2_rn(r2, bc2(c.inv_s2), bc2(1.f));
		const float2 s = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
		const float2 s2 = __fmul2_rn(s, s);
		return __fmul2_rn(__fmul2_rn(s2, s2), __fmul2_rn(s2, s));   // (1 + rho^2)^-3.5
	} };
template <> struct ZetaShape2<Reg::Planetary> {
	static constexpr double kFactor = 3.0;
	__device__ __forceinline__ static float2 z(float2 r2, const RegConsts& c) {
		return make_float2(r2.x < c.s2 ? 1.f : 0.f, r2.y < c.s2 ? 1.f : 0.f);
	} };
template <> struct ZetaShape2<Reg::Gaussian> {
	static constexpr double kFactor = 0.7978845608028654;   // sqrt(2/pi)
	__device__ __forceinline__ static float2 z(float2 r2, const RegConsts& c) {
		const float2 a = __fmul2_rn(r2, bc2(c.exp2_half));
		return make_float2(ex2_approx(a.x), ex2_approx(a.y));       // exp(-rho^2/2)
	} };


template <bool VEL, bool DV> struct InduceNC { static constexpr int value = (VEL ? 3 : 0) + (DV ? 6 : 0); };

struct InduceConsts {
	RegConsts rc;
	double s_vel, s_dv, k_scale;
};

// Output scales and regularisation constants for one regularisation distance
// (host; p3d.cu).
InduceConsts make_induce_consts(int reg, float sigma);

// Shared memory of one CTA: tile stages + barriers + (hi, lo) per target and sum.
template <int TPT, int NT, int NC, int TILE = kP3DTile>
constexpr size_t induce_smem_bytes() {
	return P3DStreamT<TILE>::kSmemBytes + size_t(2) * NC * TPT * NT * sizeof(float);
}

template <bool VEL, bool DV>
__device__ __forceinline__ void write_induce(const P3DInduceProblem& p,
	const InduceConsts& kc, int t, const double* s)
{
	int o = 0;
	if (VEL) {
		float* v = p.out_vel + 3 * size_t(t);
		v[0] = float(kc.s_vel * s[0]);
		v[1] = float(kc.s_vel * s[1]);
		v[2] = float(kc.s_vel * s[2]);
		o = 3;
	}
	if (DV) {
		float* w = p.out_dvort + 3 * size_t(t);
		w[0] = float(kc.s_dv * (s[o + 0] - kc.k_scale * s[o + 3]));
		w[1] = float(kc.s_dv * (s[o + 1] - kc.k_scale * s[o + 4]));
		w[2] = float(kc.s_dv * (s[o + 2] - kc.k_scale * s[o + 5]));
	}
}

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// co = a x b per lane, rounded as the reference rounds it: each component is
// the difference of two rounded products (nb = -b, so that the second
// product carries its sign and needs no separate negation).
__device__ __forceinline__ void cross_ref2(float2 ax, float2 ay, float2 az,
	float2 bx, float2 by, float2 bz, float2 nbx, float2 nby, float2 nbz,
	float2& cx, float2& cy, float2& cz)
{
	cx = __fadd2_rn(__fmul2_rn(ay, bz), __fmul2_rn(az, nby));
	cy = __fadd2_rn(__fmul2_rn(az, bx), __fmul2_rn(ax, nbz));
	cz = __fadd2_rn(__fmul2_rn(ax, by), __fmul2_rn(ay, nbx));
}

// Packed CTA body: targets tbase + k*NT + threadIdx.x (k < TPT; thread-local
// pairs (2h, 2h+1) share one f32x2 lane pair) against sources
// [s_begin, s_begin + n_s) streamed through `smem` (barriers initialised by
// P3DStream::init; `tcount` carries the stage phase across calls). For every
// valid target calls sink(t, sums[NC]). Returns false if the tile pipeline
// timed out (results were not produced).
template <Reg R, bool VEL, bool DV, int TPT, int NT, int UNROLL = 2, int TILE = kP3DTile,
	class Sink>
__device__ __forceinline__ bool induce2_block(const P3DInduceProblem& p, const InduceConsts& kc,
	int tbase, int s_begin, int n_s, unsigned char* smem, unsigned* err, unsigned& tcount,
	Sink&& sink)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int H = TPT / 2;
	constexpr int NC = InduceNC<VEL, DV>::value;
	constexpr int NR = NC;
	constexpr bool kFinite = FiniteAtZero<R>::value;
	using Stream = P3DStreamT<TILE>;
	float* hi = reinterpret_cast<float*>(smem + Stream::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const RegConsts rc = kc.rc;

	float2 tx[H], ty[H], tz[H], ax[H], ay[H], az[H];
#pragma unroll
	for (int h = 0; h < H; ++h) {
		float4 q[2], v[2];
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			int t = tbase + (2 * h + e) * NT + tid;
			t = t < p.n_tgt ? t : p.n_tgt - 1;
			q[e] = p.tgt[size_t(t) * p.tstride];
			v[e] = DV ? p.tgt[size_t(t) * p.tstride + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
		}
		tx[h] = make_float2(q[0].x, q[1].x); ty[h] = make_float2(q[0].y, q[1].y);
		tz[h] = make_float2(q[0].z, q[1].z);
		ax[h] = make_float2(v[0].x, v[1].x); ay[h] = make_float2(v[0].y, v[1].y);
		az[h] = make_float2(v[0].z, v[1].z);
	}
#pragma unroll
	for (int i = 0; i < NC * TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }

	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float2 acc[NR][H];
#pragma unroll
		for (int c = 0; c < NR; ++c)
#pragma unroll
			for (int h = 0; h < H; ++h) acc[c][h] = make_float2(0.f, 0.f);

		auto body = [&](int j) {
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
			const float2 sx = bc2(sp.x), sy = bc2(sp.y), sz = bc2(sp.z);
			const float2 wx = bc2(sv.x), wy = bc2(sv.y), wz = bc2(sv.z);
			const float2 nwx = bc2(-sv.x), nwy = bc2(-sv.y), nwz = bc2(-sv.z);
#pragma unroll
			for (int h = 0; h < H; ++h) {
				// d = t - s as s * (-1) + t: one rounding, no per-source negation
				const float2 dx = __ffma2_rn(sx, bc2(-1.f), tx[h]);
				const float2 dy = __ffma2_rn(sy, bc2(-1.f), ty[h]);
				const float2 dz = __ffma2_rn(sz, bc2(-1.f), tz[h]);
				const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
				// c = d x alpha_s
				const float2 cx = __ffma2_rn(dy, wz, __fmul2_rn(dz, nwy));
				const float2 cy = __ffma2_rn(dz, wx, __fmul2_rn(dx, nwz));
				const float2 cz = __ffma2_rn(dx, wy, __fmul2_rn(dy, nwx));
				if (!DV) {
					float2 G = RegP3D2<R>::g2(r2, rc);
					if (!kFinite) {
						G.x = r2.x > 0.f ? G.x : 0.f;
						G.y = r2.y > 0.f ? G.y : 0.f;
					}
					acc[0][h] = __ffma2_rn(G, cx, acc[0][h]);
					acc[1][h] = __ffma2_rn(G, cy, acc[1][h]);
					acc[2][h] = __ffma2_rn(G, cz, acc[2][h]);
					continue;
				}
				float2 G, K;
				RegP3D2<R>::gk2(r2, rc, G, K);
				G.x = r2.x > 0.f ? G.x : 0.f;
				G.y = r2.y > 0.f ? G.y : 0.f;
				if (!kFinite) {
					K.x = r2.x > 0.f ? K.x : 0.f;
					K.y = r2.y > 0.f ? K.y : 0.f;
				}
				constexpr int o = VEL ? 3 : 0;
				if (VEL) {
					acc[0][h] = __ffma2_rn(G, cx, acc[0][h]);
					acc[1][h] = __ffma2_rn(G, cy, acc[1][h]);
					acc[2][h] = __ffma2_rn(G, cz, acc[2][h]);
				}
				// co = alpha_t x alpha_s (reference rounding)
				float2 ox, oy, oz;
				cross_ref2(ax[h], ay[h], az[h], wx, wy, wz, nwx, nwy, nwz, ox, oy, oz);
				acc[o + 0][h] = __ffma2_rn(G, ox, acc[o + 0][h]);
				acc[o + 1][h] = __ffma2_rn(G, oy, acc[o + 1][h]);
				acc[o + 2][h] = __ffma2_rn(G, oz, acc[o + 2][h]);
				const float2 pd = __ffma2_rn(dz, oz, __ffma2_rn(dy, oy, __fmul2_rn(dx, ox)));
				const float2 kk = __fmul2_rn(K, pd);
				acc[o + 3][h] = __ffma2_rn(kk, dx, acc[o + 3][h]);
				acc[o + 4][h] = __ffma2_rn(kk, dy, acc[o + 4][h]);
				acc[o + 5][h] = __ffma2_rn(kk, dz, acc[o + 5][h]);
			}
		};
		if (cnt == TILE) {
#pragma unroll (UNROLL)
			for (int j = 0; j < TILE; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int c = 0; c < NC; ++c) {
#pragma unroll
			for (int h = 0; h < H; ++h) {
#pragma unroll
				for (int e = 0; e < 2; ++e) {
					const int k = 2 * h + e;
					const int i = (c * TPT + k) * NT + tid;
					float hh = hi[i], ll = lo[i];
					fold_twosum(hh, ll, e == 0 ? acc[c][h].x : acc[c][h].y);
					hi[i] = hh; lo[i] = ll;
				}
			}
		}
	};

	if (!Stream::run_continue(smem, p.src, s_begin, n_s, err, tcount, tile_fn)) return false;

#pragma unroll
	for (int h = 0; h < H; ++h) {
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			const int k = 2 * h + e;
			const int t = tbase + k * NT + tid;
			if (t >= p.n_tgt) continue;
			double sacc[NC];
#pragma unroll
			for (int c = 0; c < NC; ++c) {
				const int i = (c * TPT + k) * NT + tid;
				sacc[c] = double(hi[i]) + double(lo[i]);
			}
			sink(t, sacc);
		}
	}
	return true;
}


}  // namespace cvtx
