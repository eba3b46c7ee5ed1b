// p3d_induce.cuh -- the P3D velocity / vortex-stretching CTA body shared by
// the per-call kernels (p3d.cu) and the batched persistent kernel (batch.cu).
//
// Accumulators per target (registers, FP32, reset every tile):
//   VEL only : u  = sum G c,            c  = d x alpha_s
//   DV       : A' = sum G da,           da = alpha_s - alpha_t
//              B  = sum K (alpha_t.c') d, c' = d x da
//   VEL + DV : also u' = sum G c' and W = sum G d; since d x alpha_s =
//              c' + d x alpha_t, the velocity partial of a tile is
//              u' + W x alpha_t, formed once per tile.
// Working with da rather than alpha_s keeps the stretching terms free of the
// cancellation of nearly parallel vorticity: alpha_t x alpha_s = alpha_t x da
// and alpha_t.(d x alpha_s) = alpha_t.c' hold exactly, and da, c' are small
// when the cross products are. Per target, the compensated state across
// tiles is u (3, VEL), A' and B (6, DV), kept in shared memory as (hi, lo).
// Final outputs: vel = S_vel u, dvort = S_dv (alpha_t x A' + K_scale B).
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
	const InduceConsts& kc, int t, const double* s, float ax, float ay, float az)
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
		const double Ax = s[o], Ay = s[o + 1], Az = s[o + 2];
		const double cx = double(ay) * Az - double(az) * Ay;
		const double cy = double(az) * Ax - double(ax) * Az;
		const double cz = double(ax) * Ay - double(ay) * Ax;
		float* w = p.out_dvort + 3 * size_t(t);
		w[0] = float(kc.s_dv * (cx + kc.k_scale * s[o + 3]));
		w[1] = float(kc.s_dv * (cy + kc.k_scale * s[o + 4]));
		w[2] = float(kc.s_dv * (cz + kc.k_scale * s[o + 5]));
	}
}

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// Packed CTA body: targets tbase + k*NT + threadIdx.x (k < TPT; thread-local
// pairs (2h, 2h+1) share one f32x2 lane pair) against sources
// [s_begin, s_begin + n_s) streamed through `smem` (barriers initialised by
// P3DStream::init; `tcount` carries the stage phase across calls). For every
// valid target calls sink(t, sums[NC], alpha_t). Returns false if the tile
// pipeline timed out (results were not produced).
template <Reg R, bool VEL, bool DV, int TPT, int NT, int UNROLL = 2, int TILE = kP3DTile,
	class Sink>
__device__ __forceinline__ bool induce2_block(const P3DInduceProblem& p, const InduceConsts& kc,
	int tbase, int s_begin, int n_s, unsigned char* smem, unsigned* err, unsigned& tcount,
	Sink&& sink)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int H = TPT / 2;
	constexpr int NC = InduceNC<VEL, DV>::value;
	constexpr int NR = (VEL ? (DV ? 6 : 3) : 0) + (DV ? 6 : 0);
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
#pragma unroll
			for (int h = 0; h < H; ++h) {
				// d = t - s as s * (-1) + t: one rounding, no per-source negation
				const float2 dx = __ffma2_rn(sx, bc2(-1.f), tx[h]);
				const float2 dy = __ffma2_rn(sy, bc2(-1.f), ty[h]);
				const float2 dz = __ffma2_rn(sz, bc2(-1.f), tz[h]);
				const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
				if (!DV) {
					// c = d x alpha_s
					const float2 cx = __ffma2_rn(dy, wz, neg2(__fmul2_rn(dz, wy)));
					const float2 cy = __ffma2_rn(dz, wx, neg2(__fmul2_rn(dx, wz)));
					const float2 cz = __ffma2_rn(dx, wy, neg2(__fmul2_rn(dy, wx)));
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
				// da = alpha_s - alpha_t, c' = d x da
				const float2 ex = __ffma2_rn(ax[h], bc2(-1.f), wx);
				const float2 ey = __ffma2_rn(ay[h], bc2(-1.f), wy);
				const float2 ez = __ffma2_rn(az[h], bc2(-1.f), wz);
				const float2 cx = __ffma2_rn(dy, ez, neg2(__fmul2_rn(dz, ey)));
				const float2 cy = __ffma2_rn(dz, ex, neg2(__fmul2_rn(dx, ez)));
				const float2 cz = __ffma2_rn(dx, ey, neg2(__fmul2_rn(dy, ex)));
				float2 G, K;
				RegP3D2<R>::gk2(r2, rc, G, K);
				G.x = r2.x > 0.f ? G.x : 0.f;
				G.y = r2.y > 0.f ? G.y : 0.f;
				if (!kFinite) {
					K.x = r2.x > 0.f ? K.x : 0.f;
					K.y = r2.y > 0.f ? K.y : 0.f;
				}
				constexpr int o = VEL ? 6 : 0;
				if (VEL) {
					acc[0][h] = __ffma2_rn(G, cx, acc[0][h]);
					acc[1][h] = __ffma2_rn(G, cy, acc[1][h]);
					acc[2][h] = __ffma2_rn(G, cz, acc[2][h]);
					acc[3][h] = __ffma2_rn(G, dx, acc[3][h]);
					acc[4][h] = __ffma2_rn(G, dy, acc[4][h]);
					acc[5][h] = __ffma2_rn(G, dz, acc[5][h]);
				}
				acc[o + 0][h] = __ffma2_rn(G, ex, acc[o + 0][h]);
				acc[o + 1][h] = __ffma2_rn(G, ey, acc[o + 1][h]);
				acc[o + 2][h] = __ffma2_rn(G, ez, acc[o + 2][h]);
				const float2 pd = __ffma2_rn(az[h], cz, __ffma2_rn(ay[h], cy, __fmul2_rn(ax[h], cx)));
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
		if (VEL && DV) {
#pragma unroll
			for (int h = 0; h < H; ++h) {
				const float2 wx_ = acc[3][h], wy_ = acc[4][h], wz_ = acc[5][h];
				acc[0][h] = __fadd2_rn(acc[0][h], __ffma2_rn(wy_, az[h], neg2(__fmul2_rn(wz_, ay[h]))));
				acc[1][h] = __fadd2_rn(acc[1][h], __ffma2_rn(wz_, ax[h], neg2(__fmul2_rn(wx_, az[h]))));
				acc[2][h] = __fadd2_rn(acc[2][h], __ffma2_rn(wx_, ay[h], neg2(__fmul2_rn(wy_, ax[h]))));
			}
		}
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int src_c = (VEL && DV && c >= 3) ? c + 3 : c;
#pragma unroll
			for (int h = 0; h < H; ++h) {
#pragma unroll
				for (int e = 0; e < 2; ++e) {
					const int k = 2 * h + e;
					const int i = (c * TPT + k) * NT + tid;
					float hh = hi[i], ll = lo[i];
					fold_twosum(hh, ll, e == 0 ? acc[src_c][h].x : acc[src_c][h].y);
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
			const float tax = e == 0 ? ax[h].x : ax[h].y;
			const float tay = e == 0 ? ay[h].x : ay[h].y;
			const float taz = e == 0 ? az[h].x : az[h].y;
			sink(t, sacc, tax, tay, taz);
		}
	}
	return true;
}


}  // namespace cvtx
