// f3d.cu -- straight singular vortex filament kernels for sm_103a.
//
// Replaces cvtx_nb_Filament_ind_{vel,vel_smes,dvort}_singular (reference
// src/nbody.cl:611-728) and src/ocl_F3D.cpp. Per-pair arithmetic follows the
// reference CPU path src/F3D.cpp:34-54 (velocity), :56-85 (vortex
// stretching) and :204-227 (influence matrix), including its guards: a
// velocity term is dropped when |t1| or |t2| exceeds FLT_MAX (or is NaN), a
// stretching term when it contains NaN. For stretching the 1/(4 pi) factor is
// applied once per target.
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include "nbody.h"
#include "plan.cuh"
#include "regfuncs.cuh"
#include "tile_stream.cuh"
#include "few.cuh"

namespace cvtx {
namespace {

constexpr int kTile = 256;
constexpr int kStages = 2;
using Stream2 = TileStream<2, kTile, kStages>;
constexpr int kSmallTargets = 8192;
constexpr double kInv4Pi = 1.0 / (4.0 * 3.14159265358979323846);
constexpr float kBig = 3.40282346e38f;
constexpr float kInv4PiF = float(kInv4Pi);

// The reference's straight-segment factor t2 / |r1 x r2|^2 with
// t2 = r0.r1/|r1| - r0.r2/|r2| (src/F3D.cpp:34-54), r1 = m - s, r2 = m - e,
// r0 = r1 - r2, in whichever of two exact rewritings has no cancellation
// for the pair (with q = |r|^2, d = r1.r2, l = |r|):
//   d < 0:  t2 = (q1 - d)/l1 + (q2 - d)/l2           over |r1 x r2|^2
//   d >= 0: t2 / |r1 x r2|^2 = (l1 + l2) / (l1 l2 (l1 l2 + d))
// (|r1 x r2|^2 = (l1 l2 - d)(l1 l2 + d)). The reference's own form cancels
// where the point is far from the segment or near the line beyond its ends,
// which costs it up to about 1e-4 relative accuracy on single terms; these
// forms keep every term to a few ulp. Returns the numerator and denominator;
// the caller divides and drops the term when the quotient is not finite (a
// point on the segment or at an end point, where the reference's term is
// infinite or NaN and dropped too).
__device__ __forceinline__ void f3d_factor(float q1, float q2, float d, float il1, float il2,
	float cc, float& num, float& den)
{
	const float l1 = q1 * il1, l2 = q2 * il2;
	const float L = l1 * l2;
	const bool inner = d < 0.f;
	num = inner ? fmaf(q1 - d, il1, (q2 - d) * il2) : l1 + l2;
	den = inner ? cc : L * (L + d);
}

// Velocity induced at m by filament (s -> e) of strength gamma, including the
// 1/(4 pi) factor (reference src/F3D.cpp:34-54); a term whose factor is not
// finite is dropped, as the reference drops it.
__device__ __forceinline__ void f3d_vel_pair(float mx, float my, float mz,
	const float4 a, const float4 b, float& vx, float& vy, float& vz)
{
	const float r1x = mx - a.x, r1y = my - a.y, r1z = mz - a.z;
	const float r2x = mx - b.x, r2y = my - b.y, r2z = mz - b.z;
	const float cx = fmaf(r1y, r2z, -r1z * r2y);
	const float cy = fmaf(r1z, r2x, -r1x * r2z);
	const float cz = fmaf(r1x, r2y, -r1y * r2x);
	const float cc = fmaf(cz, cz, fmaf(cy, cy, cx * cx));
	const float q1 = fmaf(r1z, r1z, fmaf(r1y, r1y, r1x * r1x));
	const float q2 = fmaf(r2z, r2z, fmaf(r2y, r2y, r2x * r2x));
	const float d = fmaf(r1z, r2z, fmaf(r1y, r2y, r1x * r2x));
	float num, den;
	f3d_factor(q1, q2, d, rsqrt_approx(q1), rsqrt_approx(q2), cc, num, den);
	const float f = (a.w * kInv4PiF) * num / den;
	// |f| <= FLT_MAX; NaN fails
	const bool ok = fabsf(f) <= kBig;
	vx = ok ? cx * f : 0.f;
	vy = ok ? cy * f : 0.f;
	vz = ok ? cz * f : 0.f;
}

template <int TPT, int NT>
__global__ void __launch_bounds__(NT)
f3d_vel_kernel(const F3DVelProblem p, double* __restrict__ partial, int src_per_split,
	unsigned* err)
{
	constexpr int NC = 3;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_fil - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float tx[TPT], ty[TPT], tz[TPT];
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		int t = tbase + k * NT + tid;
		t = t < p.n_tgt ? t : p.n_tgt - 1;
		const float4 tp = p.tgt[size_t(t) * p.tstride];
		tx[k] = tp.x; ty[k] = tp.y; tz[k] = tp.z;
	}
#pragma unroll
	for (int i = 0; i < NC * TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }
	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float acc[NC][TPT];
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int k = 0; k < TPT; ++k) acc[c][k] = 0.f;
		auto body = [&](int j) {
			const float4 a = st[2 * j];
			const float4 b = st[2 * j + 1];
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				float vx, vy, vz;
				f3d_vel_pair(tx[k], ty[k], tz[k], a, b, vx, vy, vz);
				acc[0][k] += vx; acc[1][k] += vy; acc[2][k] += vz;
			}
		};
		if (cnt == kTile) {
#pragma unroll 2
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const int i = (c * TPT + k) * NT + tid;
				float h = hi[i], l = lo[i];
				fold_twosum(h, l, acc[c][k]);
				hi[i] = h; lo[i] = l;
			}
	};
	if (!Stream2::run(smem, p.fil, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

__device__ __forceinline__ float2 neg2f(float2 a) { return make_float2(-a.x, -a.y); }

// f3d_factor for two points at once (per lane). Where no pair of the warp's
// live lanes lies beside its segment (d >= 0 everywhere: beyond the ends or
// far away, most pairs of a sheet), only the product form is evaluated; the
// result is the same as with the per-pair select. (Timed on a GB300: wake
// sheet velocity, 50,000 x 50,000, 673 -> 782 G/s; stretching, 100,000 x
// 100,000, 518 -> 571 G/s; influence matrix 25,000 x 20,000: 0.818 ->
// 0.783 ms.)
__device__ __forceinline__ void f3d_factor2(float2 q1, float2 q2, float2 d, float2 il1,
	float2 il2, float2 cc, float2& num, float2& den)
{
	const float2 l1 = __fmul2_rn(q1, il1), l2 = __fmul2_rn(q2, il2);
	const float2 L = __fmul2_rn(l1, l2);
	if (!__any_sync(__activemask(), d.x < 0.f || d.y < 0.f)) {
		num = __fadd2_rn(l1, l2);
		den = __fmul2_rn(L, __fadd2_rn(L, d));
		return;
	}
	const float2 nd = neg2f(d);
	const float2 na = __ffma2_rn(__fadd2_rn(q1, nd), il1, __fmul2_rn(__fadd2_rn(q2, nd), il2));
	const float2 nb = __fadd2_rn(l1, l2);
	const float2 db = __fmul2_rn(L, __fadd2_rn(L, d));
	num = make_float2(d.x < 0.f ? na.x : nb.x, d.y < 0.f ? na.y : nb.y);
	den = make_float2(d.x < 0.f ? cc.x : db.x, d.y < 0.f ? cc.y : db.y);
}

// f3d_vel_pair for two measurement points at once (f32x2), with the
// division done as a reciprocal refined by one Newton step; same guard.
__device__ __forceinline__ void f3d_vel_pair2(float2 mx, float2 my, float2 mz,
	const float4 a, const float4 b, float2& vx, float2& vy, float2& vz)
{
	const float2 r1x = __fadd2_rn(mx, bc2(-a.x)), r1y = __fadd2_rn(my, bc2(-a.y));
	const float2 r1z = __fadd2_rn(mz, bc2(-a.z));
	const float2 r2x = __fadd2_rn(mx, bc2(-b.x)), r2y = __fadd2_rn(my, bc2(-b.y));
	const float2 r2z = __fadd2_rn(mz, bc2(-b.z));
	const float2 cx = __ffma2_rn(r1y, r2z, neg2f(__fmul2_rn(r1z, r2y)));
	const float2 cy = __ffma2_rn(r1z, r2x, neg2f(__fmul2_rn(r1x, r2z)));
	const float2 cz = __ffma2_rn(r1x, r2y, neg2f(__fmul2_rn(r1y, r2x)));
	const float2 cc = __ffma2_rn(cz, cz, __ffma2_rn(cy, cy, __fmul2_rn(cx, cx)));
	const float2 q1 = __ffma2_rn(r1z, r1z, __ffma2_rn(r1y, r1y, __fmul2_rn(r1x, r1x)));
	const float2 q2 = __ffma2_rn(r2z, r2z, __ffma2_rn(r2y, r2y, __fmul2_rn(r2x, r2x)));
	const float2 d = __ffma2_rn(r1z, r2z, __ffma2_rn(r1y, r2y, __fmul2_rn(r1x, r2x)));
	const float2 il1 = make_float2(rsqrt_approx(q1.x), rsqrt_approx(q1.y));
	const float2 il2 = make_float2(rsqrt_approx(q2.x), rsqrt_approx(q2.y));
	float2 num, den;
	f3d_factor2(q1, q2, d, il1, il2, cc, num, den);
	const float2 f = __fmul2_rn(__fmul2_rn(bc2(a.w * kInv4PiF), num), rcp2(den));
	const bool okx = fabsf(f.x) <= kBig;
	const bool oky = fabsf(f.y) <= kBig;
	vx = __fmul2_rn(cx, f);
	vy = __fmul2_rn(cy, f);
	vz = __fmul2_rn(cz, f);
	// a dropped term is exactly zero even where c is not finite
	if (!okx) { vx.x = 0.f; vy.x = 0.f; vz.x = 0.f; }
	if (!oky) { vx.y = 0.f; vy.y = 0.f; vz.y = 0.f; }
}

template <int TPT, int NT>
__global__ void __launch_bounds__(NT)
f3d_vel2_kernel(const F3DVelProblem p, double* __restrict__ partial, int src_per_split,
	unsigned* err)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int NC = 3, H = TPT / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_fil - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float2 tx[H], ty[H], tz[H];
#pragma unroll
	for (int h = 0; h < H; ++h) {
		float4 q[2];
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			int t = tbase + (2 * h + e) * NT + tid;
			t = t < p.n_tgt ? t : p.n_tgt - 1;
			q[e] = p.tgt[size_t(t) * p.tstride];
		}
		tx[h] = make_float2(q[0].x, q[1].x);
		ty[h] = make_float2(q[0].y, q[1].y);
		tz[h] = make_float2(q[0].z, q[1].z);
	}
#pragma unroll
	for (int i = 0; i < NC * TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }
	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float2 acc[NC][H];
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int h = 0; h < H; ++h) acc[c][h] = make_float2(0.f, 0.f);
		auto body = [&](int j) {
			const float4 a = st[2 * j];
			const float4 b = st[2 * j + 1];
#pragma unroll
			for (int h = 0; h < H; ++h) {
				float2 vx, vy, vz;
				f3d_vel_pair2(tx[h], ty[h], tz[h], a, b, vx, vy, vz);
				acc[0][h] = __fadd2_rn(acc[0][h], vx);
				acc[1][h] = __fadd2_rn(acc[1][h], vy);
				acc[2][h] = __fadd2_rn(acc[2][h], vz);
			}
		};
		if (cnt == kTile) {
#pragma unroll 2
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int h = 0; h < H; ++h)
#pragma unroll
				for (int e = 0; e < 2; ++e) {
					const int i = (c * TPT + 2 * h + e) * NT + tid;
					float hv = hi[i], lv = lo[i];
					fold_twosum(hv, lv, e == 0 ? acc[c][h].x : acc[c][h].y);
					hi[i] = hv; lo[i] = lv;
				}
	};
	if (!Stream2::run(smem, p.fil, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

// Vortex stretching of particle (x, alpha) by filament (s -> e), strength g,
// without the 1/(4 pi) factor (reference src/F3D.cpp:56-85):
//   r1 = x - s, r2 = x - e, r0 = r1 - r2, X = |r1 x r0| (= |r1 x r2|)
//   A = -r0 / X^2 * g * (r0.r1/|r1| - r0.r2/|r2|)
//   B = 3/|r0| * g * (X/|r1| - X/|r2|)
//   out = B alpha + A x alpha
// The factor of A is the velocity factor t2 / X^2, evaluated as f3d_factor
// does. A particle exactly on the filament's line (X = 0), where the
// reference's term is infinite or NaN, has its term dropped, as has any term
// that is not finite.
__device__ __forceinline__ void f3d_dvort_pair(float px, float py, float pz,
	float wx, float wy, float wz, const float4 a, const float4 b,
	float& ox, float& oy, float& oz)
{
	const float r1x = px - a.x, r1y = py - a.y, r1z = pz - a.z;
	const float r2x = px - b.x, r2y = py - b.y, r2z = pz - b.z;
	const float r0x = r1x - r2x, r0y = r1y - r2y, r0z = r1z - r2z;
	const float xx = fmaf(r1y, r0z, -r1z * r0y);
	const float xy = fmaf(r1z, r0x, -r1x * r0z);
	const float xz = fmaf(r1x, r0y, -r1y * r0x);
	const float X2 = fmaf(xz, xz, fmaf(xy, xy, xx * xx));
	const float X = sqrtf(X2);
	const float q1 = fmaf(r1z, r1z, fmaf(r1y, r1y, r1x * r1x));
	const float q2 = fmaf(r2z, r2z, fmaf(r2y, r2y, r2x * r2x));
	const float d = fmaf(r1z, r2z, fmaf(r1y, r2y, r1x * r2x));
	const float il1 = rsqrt_approx(q1);
	const float il2 = rsqrt_approx(q2);
	const float il0 = rsqrt_approx(fmaf(r0z, r0z, fmaf(r0y, r0y, r0x * r0x)));
	float num, den;
	f3d_factor(q1, q2, d, il1, il2, X2, num, den);
	const float kA = -a.w * num / den;
	const float Ax = r0x * kA, Ay = r0y * kA, Az = r0z * kA;
	const float t222 = X * il1 - X * il2;
	const float B = 3.f * il0 * a.w * t222;
	const float vx = fmaf(wx, B, fmaf(Ay, wz, -Az * wy));
	const float vy = fmaf(wy, B, fmaf(Az, wx, -Ax * wz));
	const float vz = fmaf(wz, B, fmaf(Ax, wy, -Ay * wx));
	const bool ok = X2 > 0.f && fabsf(vx) <= kBig && fabsf(vy) <= kBig && fabsf(vz) <= kBig;
	ox = ok ? vx : 0.f;
	oy = ok ? vy : 0.f;
	oz = ok ? vz : 0.f;
}

// f3d_dvort_pair for two particles at once (f32x2). `c` holds what depends
// on the filament alone, computed once per staged tile: r0 = e - s (the
// reference forms r1 - r2 per pair; the two differ by rounding) and
// 3 g / |r0|. |r1 x r0| comes from X2 * rsqrt(X2); the factor of A from
// f3d_factor2 with a Newton-refined reciprocal.
__device__ __forceinline__ void f3d_dvort_pair2(float2 px, float2 py, float2 pz,
	float2 wx, float2 wy, float2 wz, const float4 a, const float4 b, const float4 c,
	float2& ox, float2& oy, float2& oz)
{
	const float2 r1x = __fadd2_rn(px, bc2(-a.x)), r1y = __fadd2_rn(py, bc2(-a.y));
	const float2 r1z = __fadd2_rn(pz, bc2(-a.z));
	const float2 r2x = __fadd2_rn(px, bc2(-b.x)), r2y = __fadd2_rn(py, bc2(-b.y));
	const float2 r2z = __fadd2_rn(pz, bc2(-b.z));
	const float2 r0x = bc2(c.x), r0y = bc2(c.y), r0z = bc2(c.z);
	const float2 xx = __ffma2_rn(r1y, r0z, neg2f(__fmul2_rn(r1z, r0y)));
	const float2 xy = __ffma2_rn(r1z, r0x, neg2f(__fmul2_rn(r1x, r0z)));
	const float2 xz = __ffma2_rn(r1x, r0y, neg2f(__fmul2_rn(r1y, r0x)));
	const float2 X2 = __ffma2_rn(xz, xz, __ffma2_rn(xy, xy, __fmul2_rn(xx, xx)));
	const float2 iX = make_float2(rsqrt_approx(X2.x), rsqrt_approx(X2.y));
	const float2 X = __fmul2_rn(X2, iX);
	const float2 q1 = __ffma2_rn(r1z, r1z, __ffma2_rn(r1y, r1y, __fmul2_rn(r1x, r1x)));
	const float2 q2 = __ffma2_rn(r2z, r2z, __ffma2_rn(r2y, r2y, __fmul2_rn(r2x, r2x)));
	const float2 d = __ffma2_rn(r1z, r2z, __ffma2_rn(r1y, r2y, __fmul2_rn(r1x, r2x)));
	const float2 il1 = make_float2(rsqrt_approx(q1.x), rsqrt_approx(q1.y));
	const float2 il2 = make_float2(rsqrt_approx(q2.x), rsqrt_approx(q2.y));
	float2 num, den;
	f3d_factor2(q1, q2, d, il1, il2, X2, num, den);
	const float2 t222 = __fmul2_rn(X, __fadd2_rn(il1, neg2f(il2)));
	const float2 kA = __fmul2_rn(__fmul2_rn(bc2(-a.w), num), rcp2(den));
	const float2 Ax = __fmul2_rn(r0x, kA), Ay = __fmul2_rn(r0y, kA), Az = __fmul2_rn(r0z, kA);
	const float2 B = __fmul2_rn(bc2(c.w), t222);
	const float2 vx = __ffma2_rn(wx, B, __ffma2_rn(Ay, wz, neg2f(__fmul2_rn(Az, wy))));
	const float2 vy = __ffma2_rn(wy, B, __ffma2_rn(Az, wx, neg2f(__fmul2_rn(Ax, wz))));
	const float2 vz = __ffma2_rn(wz, B, __ffma2_rn(Ax, wy, neg2f(__fmul2_rn(Ay, wx))));
	const bool okx = X2.x > 0.f && fabsf(vx.x) <= kBig && fabsf(vy.x) <= kBig &&
		fabsf(vz.x) <= kBig;
	const bool oky = X2.y > 0.f && fabsf(vx.y) <= kBig && fabsf(vy.y) <= kBig &&
		fabsf(vz.y) <= kBig;
	ox = make_float2(okx ? vx.x : 0.f, oky ? vx.y : 0.f);
	oy = make_float2(okx ? vy.x : 0.f, oky ? vy.y : 0.f);
	oz = make_float2(okx ? vz.x : 0.f, oky ? vz.y : 0.f);
}

template <int TPT, int NT>
__global__ void __launch_bounds__(NT)
f3d_dvort2_kernel(const F3DDvortProblem p, double* __restrict__ partial, int src_per_split,
	unsigned* err)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int NC = 3, H = TPT / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	float4* fil_c = reinterpret_cast<float4*>(lo + NC * TPT * NT);   // kTile per-filament terms
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_fil - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float2 tx[H], ty[H], tz[H], ax[H], ay[H], az[H];
#pragma unroll
	for (int h = 0; h < H; ++h) {
		float4 q[2], v[2];
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			int t = tbase + (2 * h + e) * NT + tid;
			t = t < p.n_tgt ? t : p.n_tgt - 1;
			q[e] = p.tgt[size_t(t) * p.tstride];
			v[e] = p.tgt[size_t(t) * p.tstride + 1];
		}
		tx[h] = make_float2(q[0].x, q[1].x); ty[h] = make_float2(q[0].y, q[1].y);
		tz[h] = make_float2(q[0].z, q[1].z);
		ax[h] = make_float2(v[0].x, v[1].x); ay[h] = make_float2(v[0].y, v[1].y);
		az[h] = make_float2(v[0].z, v[1].z);
	}
#pragma unroll
	for (int i = 0; i < NC * TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }
	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float2 acc[NC][H];
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int h = 0; h < H; ++h) acc[c][h] = make_float2(0.f, 0.f);
		// the previous tile's readers are done (the stream synchronises the
		// CTA after every tile), so the table is rewritten here
		for (int j = tid; j < cnt; j += NT) {
			const float4 a = st[2 * j], b = st[2 * j + 1];
			const float r0x = b.x - a.x, r0y = b.y - a.y, r0z = b.z - a.z;
			const float l0 = sqrtf(fmaf(r0z, r0z, fmaf(r0y, r0y, r0x * r0x)));
			fil_c[j] = make_float4(r0x, r0y, r0z, (3.f / l0) * a.w);
		}
		__syncthreads();
		auto body = [&](int j) {
			const float4 a = st[2 * j];
			const float4 b = st[2 * j + 1];
			const float4 fc = fil_c[j];
#pragma unroll
			for (int h = 0; h < H; ++h) {
				float2 vx, vy, vz;
				f3d_dvort_pair2(tx[h], ty[h], tz[h], ax[h], ay[h], az[h], a, b, fc, vx, vy, vz);
				acc[0][h] = __fadd2_rn(acc[0][h], vx);
				acc[1][h] = __fadd2_rn(acc[1][h], vy);
				acc[2][h] = __fadd2_rn(acc[2][h], vz);
			}
		};
		if (cnt == kTile) {
#pragma unroll 2
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int h = 0; h < H; ++h)
#pragma unroll
				for (int e = 0; e < 2; ++e) {
					const int i = (c * TPT + 2 * h + e) * NT + tid;
					float hv = hi[i], lv = lo[i];
					fold_twosum(hv, lv, e == 0 ? acc[c][h].x : acc[c][h].y);
					hi[i] = hv; lo[i] = lv;
				}
	};
	if (!Stream2::run(smem, p.fil, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(kInv4Pi * s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

template <int TPT, int NT>
__global__ void __launch_bounds__(NT)
f3d_dvort_kernel(const F3DDvortProblem p, double* __restrict__ partial, int src_per_split,
	unsigned* err)
{
	constexpr int NC = 3;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_fil - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float tx[TPT], ty[TPT], tz[TPT], ax[TPT], ay[TPT], az[TPT];
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		int t = tbase + k * NT + tid;
		t = t < p.n_tgt ? t : p.n_tgt - 1;
		const float4 tp = p.tgt[size_t(t) * p.tstride];
		const float4 tv = p.tgt[size_t(t) * p.tstride + 1];
		tx[k] = tp.x; ty[k] = tp.y; tz[k] = tp.z;
		ax[k] = tv.x; ay[k] = tv.y; az[k] = tv.z;
	}
#pragma unroll
	for (int i = 0; i < NC * TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }
	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float acc[NC][TPT];
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int k = 0; k < TPT; ++k) acc[c][k] = 0.f;
		auto body = [&](int j) {
			const float4 a = st[2 * j];
			const float4 b = st[2 * j + 1];
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				float vx, vy, vz;
				f3d_dvort_pair(tx[k], ty[k], tz[k], ax[k], ay[k], az[k], a, b, vx, vy, vz);
				acc[0][k] += vx; acc[1][k] += vy; acc[2][k] += vz;
			}
		};
		if (cnt == kTile) {
#pragma unroll 2
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int c = 0; c < NC; ++c)
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const int i = (c * TPT + k) * NT + tid;
				float h = hi[i], l = lo[i];
				fold_twosum(h, l, acc[c][k]);
				hi[i] = h; lo[i] = l;
			}
	};
	if (!Stream2::run(smem, p.fil, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(kInv4Pi * s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

__global__ void f3d_finalize(float* __restrict__ out, int n_tgt,
	const double* __restrict__ partial, int n_split, double scale)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n_tgt) return;
	double s0 = 0.0, s1 = 0.0, s2 = 0.0;
	for (int sp = 0; sp < n_split; ++sp) {
		s0 += partial[(size_t(sp) * 3 + 0) * n_tgt + t];
		s1 += partial[(size_t(sp) * 3 + 1) * n_tgt + t];
		s2 += partial[(size_t(sp) * 3 + 2) * n_tgt + t];
	}
	out[3 * size_t(t) + 0] = float(scale * s0);
	out[3 * size_t(t) + 1] = float(scale * s1);
	out[3 * size_t(t) + 2] = float(scale * s2);
}

// Influence matrix: out[i * n_fil + j] = dot(vel_j(mes_i), dir_i).
// Output-write bound: each work item is a run of 4 consecutive filaments of
// one row (one 16-byte store when aligned); a grid-stride loop over the
// n_mes * ceil(n_fil / 4) items uses 64-bit indices.
__global__ void f3d_inf_kernel(const F3DInfProblem p)
{
	const long long per_row = (p.n_fil + 3) / 4;
	const long long items = per_row * p.n_mes;
	for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < items;
		w += (long long)gridDim.x * blockDim.x) {
		const int i = int(w / per_row);
		const int j0 = int(w - (long long)i * per_row) * 4;
		const float4 m = p.mes[i];
		const float4 d = p.dir[i];
		float r[4];
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			const int j = j0 + q;
			r[q] = 0.f;
			if (j < p.n_fil) {
				const float4 a = __ldg(&p.fil[2 * size_t(j)]);
				const float4 b = __ldg(&p.fil[2 * size_t(j) + 1]);
				float vx, vy, vz;
				f3d_vel_pair(m.x, m.y, m.z, a, b, vx, vy, vz);
				r[q] = fmaf(vz, d.z, fmaf(vy, d.y, vx * d.x));
			}
		}
		float* row = p.out + size_t(i) * p.n_fil;
		if (j0 + 3 < p.n_fil && ((reinterpret_cast<uintptr_t>(row + j0) & 15u) == 0)) {
			*reinterpret_cast<float4*>(row + j0) = make_float4(r[0], r[1], r[2], r[3]);
		} else {
#pragma unroll
			for (int q = 0; q < 4; ++q) if (j0 + q < p.n_fil) row[j0 + q] = r[q];
		}
	}
}

// Tiled influence matrix: a CTA covers 16 PAIRS points x kInfFils filaments;
// the filament tile sits in shared memory, and each thread evaluates PAIRS
// pairs of points (f32x2) against four consecutive filaments held in
// registers, storing float4 runs, so a warp writes 512 contiguous bytes of
// each of its rows. All lanes of a warp share their points (broadcast loads).
constexpr int kInfFils = 128;                 // 32 threads x 4 filaments
constexpr int kInfThreads = 256;
template <int PAIRS> constexpr int inf_rows() { return 8 * 2 * PAIRS; }

// One influence entry per lane: dir . (velocity of filament a -> b at m), the
// terms of f3d_vel_pair2 with the direction dotted in before the guard, so
// one test and one select drop a non-finite term. ga = gamma / (4 pi).
// Differences are formed as fma(x, -1, y): one rounding, as y - x.
// One filament's operands, each held twice (one per point of a lane pair).
struct InfFil2 { float2 ax, ay, az, bx, by, bz, ga; };

__device__ __forceinline__ float2 f3d_inf_pair2(float2 mx, float2 my, float2 mz,
	float2 ex, float2 ey, float2 ez, const InfFil2& f2)
{
	const float2 m1 = bc2(-1.f);
	const float2 r1x = __ffma2_rn(f2.ax, m1, mx), r1y = __ffma2_rn(f2.ay, m1, my);
	const float2 r1z = __ffma2_rn(f2.az, m1, mz);
	const float2 r2x = __ffma2_rn(f2.bx, m1, mx), r2y = __ffma2_rn(f2.by, m1, my);
	const float2 r2z = __ffma2_rn(f2.bz, m1, mz);
	const float2 cx = __ffma2_rn(r1y, r2z, neg2f(__fmul2_rn(r1z, r2y)));
	const float2 cy = __ffma2_rn(r1z, r2x, neg2f(__fmul2_rn(r1x, r2z)));
	const float2 cz = __ffma2_rn(r1x, r2y, neg2f(__fmul2_rn(r1y, r2x)));
	const float2 cc = __ffma2_rn(cz, cz, __ffma2_rn(cy, cy, __fmul2_rn(cx, cx)));
	const float2 q1 = __ffma2_rn(r1z, r1z, __ffma2_rn(r1y, r1y, __fmul2_rn(r1x, r1x)));
	const float2 q2 = __ffma2_rn(r2z, r2z, __ffma2_rn(r2y, r2y, __fmul2_rn(r2x, r2x)));
	const float2 d = __ffma2_rn(r1z, r2z, __ffma2_rn(r1y, r2y, __fmul2_rn(r1x, r2x)));
	const float2 il1 = make_float2(rsqrt_approx(q1.x), rsqrt_approx(q1.y));
	const float2 il2 = make_float2(rsqrt_approx(q2.x), rsqrt_approx(q2.y));
	float2 num, den;
	f3d_factor2(q1, q2, d, il1, il2, cc, num, den);
	const float2 f = __fmul2_rn(__fmul2_rn(f2.ga, num), rcp2(den));
	const float2 cd = __ffma2_rn(cz, ez, __ffma2_rn(cy, ey, __fmul2_rn(cx, ex)));
	float2 r = __fmul2_rn(f, cd);
	// |f| <= FLT_MAX; NaN fails
	r.x = fabsf(f.x) <= kBig ? r.x : 0.f;
	r.y = fabsf(f.y) <= kBig ? r.y : 0.f;
	return r;
}

template <int PAIRS, int UNROLL>
__global__ void __launch_bounds__(kInfThreads) f3d_inf2_kernel(const F3DInfProblem p)
{
	constexpr int kInfRows = inf_rows<PAIRS>();
	__shared__ float4 fs[2 * kInfFils];
	const int tx = threadIdx.x & 31;          // filament quad
	const int ty = threadIdx.x >> 5;          // point-pair lane
	const int j_base = blockIdx.y * kInfFils;
	for (int k = threadIdx.x; k < 2 * kInfFils; k += kInfThreads) {
		const int j = j_base + (k >> 1);
		fs[k] = j < p.n_fil ? p.fil[2 * size_t(j) + (k & 1)] : make_float4(0.f, 0.f, 0.f, 0.f);
	}
	__syncthreads();
	const int j0 = j_base + 4 * tx;
	if (j0 >= p.n_fil) return;
	InfFil2 fil[4];
#pragma unroll
	for (int q = 0; q < 4; ++q) {
		const float4 a = fs[2 * (4 * tx + q)], b = fs[2 * (4 * tx + q) + 1];
		fil[q].ax = bc2(a.x); fil[q].ay = bc2(a.y); fil[q].az = bc2(a.z);
		fil[q].bx = bc2(b.x); fil[q].by = bc2(b.y); fil[q].bz = bc2(b.z);
		fil[q].ga = bc2(a.w * kInv4PiF);
	}
	const bool vec = (p.n_fil & 3) == 0 && j0 + 3 < p.n_fil &&
		(reinterpret_cast<uintptr_t>(p.out) & 15u) == 0;
	// rows i0, i0 + 1 of iteration k: i0 = base + 2 (ty + 8 k); the next
	// pair's points and directions are loaded while this pair is evaluated
	const long long base = (long long)blockIdx.x * kInfRows;
	long long i0 = base + 2 * ty;
	if (i0 >= p.n_mes) return;
	auto load = [&](long long i, float4& ma, float4& mb, float4& da, float4& db) {
		const int ia = int(i);
		const int ib = int(i + 1 < p.n_mes ? i + 1 : i);
		ma = p.mes[ia]; mb = p.mes[ib];
		da = p.dir[ia]; db = p.dir[ib];
	};
	float4 ma, mb, da, db;
	load(i0, ma, mb, da, db);
#pragma unroll (UNROLL)
	for (int k = 0; k < PAIRS; ++k) {
		const long long in = i0 + 16;
		const bool more = k + 1 < PAIRS && in < p.n_mes;
		float4 na = ma, nb = mb, nda = da, ndb = db;
		if (more) load(in, na, nb, nda, ndb);
		float v2[2][4];   // [row][filament]
		const float2 mx = make_float2(ma.x, mb.x), my = make_float2(ma.y, mb.y);
		const float2 mz = make_float2(ma.z, mb.z);
		const float2 ex = make_float2(da.x, db.x), ey = make_float2(da.y, db.y);
		const float2 ez = make_float2(da.z, db.z);
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			const float2 r = f3d_inf_pair2(mx, my, mz, ex, ey, ez, fil[q]);
			v2[0][q] = r.x; v2[1][q] = r.y;
		}
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			if (e == 1 && i0 + 1 >= p.n_mes) break;
			float* row = p.out + size_t(i0 + e) * p.n_fil;
			const float* v = v2[e];
			if (vec) {
				*reinterpret_cast<float4*>(row + j0) = make_float4(v[0], v[1], v[2], v[3]);
			} else {
#pragma unroll
				for (int q = 0; q < 4; ++q) if (j0 + q < p.n_fil) row[j0 + q] = v[q];
			}
		}
		if (!more) break;
		i0 = in;
		ma = na; mb = nb; da = nda; db = ndb;
	}
}

template <int TPT, int NT>
constexpr size_t smem_bytes() {
	return Stream2::kSmemBytes + size_t(2) * 3 * TPT * NT * sizeof(float);
}

template <int TPT, int NT, bool PK>
auto vel_kernel() {
	if constexpr (PK) return f3d_vel2_kernel<TPT, NT>;
	else return f3d_vel_kernel<TPT, NT>;
}

template <int TPT, int NT, bool PK>
Plan plan_vel(int n_fil, int n_tgt, int num_sms, int max_split = 64, int min_split = 1) {
	constexpr size_t smem = smem_bytes<TPT, NT>();
	static const int occ = resident_ctas(vel_kernel<TPT, NT, PK>(), NT, smem);
	return make_plan(n_fil, n_tgt, TPT * NT, kTile, 3, num_sms * occ, smem, max_split, min_split);
}
template <int TPT, int NT, bool PK>
auto dvort_kernel() {
	if constexpr (PK) return f3d_dvort2_kernel<TPT, NT>;
	else return f3d_dvort_kernel<TPT, NT>;
}

template <int TPT, int NT, bool PK>
Plan plan_dvort(int n_fil, int n_tgt, int num_sms, int max_split = 64) {
	// the packed kernel keeps a table of kTile per-filament terms
	constexpr size_t smem = smem_bytes<TPT, NT>() + (PK ? size_t(kTile) * sizeof(float4) : 0);
	static const int occ = resident_ctas(dvort_kernel<TPT, NT, PK>(), NT, smem);
	return make_plan(n_fil, n_tgt, TPT * NT, kTile, 3, num_sms * occ, smem, max_split);
}

template <int TPT, int NT, bool PK>
cudaError_t launch_vel(const F3DVelProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_vel<TPT, NT, PK>(p.n_fil, p.n_tgt, env.num_sms,
		env.cap_to_ws ? split_cap_for(env.ws_bytes, 3, p.n_tgt) : 64, min_split_for(env, p.n_fil));
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	double* partial = static_cast<double*>(env.ws);
	vel_kernel<TPT, NT, PK>()<<<dim3(pl.n_tblocks, pl.n_split), NT, pl.smem, env.stream>>>(
		p, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		f3d_finalize<<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(p.out, p.n_tgt, partial, pl.n_split, 1.0);
		count_launch();
	}
	return cudaGetLastError();
}
template <int TPT, int NT, bool PK>
cudaError_t launch_dvort(const F3DDvortProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_dvort<TPT, NT, PK>(p.n_fil, p.n_tgt, env.num_sms,
		env.cap_to_ws ? split_cap_for(env.ws_bytes, 3, p.n_tgt) : 64);
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	double* partial = static_cast<double*>(env.ws);
	dvort_kernel<TPT, NT, PK>()<<<dim3(pl.n_tblocks, pl.n_split), NT, pl.smem, env.stream>>>(
		p, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		f3d_finalize<<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(p.out, p.n_tgt, partial, pl.n_split, kInv4Pi);
		count_launch();
	}
	return cudaGetLastError();
}

}  // namespace

// The F3D velocity pair as an operation of the few-target form (few.cuh):
// the same per-pair arithmetic as f3d_vel_kernel (f3d_vel_pair).
struct F3DVelOp {
	using Problem = F3DVelProblem;
	struct Consts { int unused; };
	static constexpr int NC = 3, NR = 3;
	struct Tgt { float x, y, z; };
	struct Src { float4 a, b; };
	__device__ static int n_src(const Problem& p) { return p.n_fil; }
	__device__ static int n_tgt(const Problem& p) { return p.n_tgt; }
	__device__ static Tgt target(const Problem& p, int t) {
		const float4 q = p.tgt[size_t(t) * p.tstride];
		return Tgt{q.x, q.y, q.z};
	}
	__device__ static Src source(const Problem& p, long long s) {
		return Src{p.fil[2 * s], p.fil[2 * s + 1]};
	}
	__device__ static void pair(const Consts&, const Tgt& t, const Src& s, float (&acc)[NR]) {
		float vx, vy, vz;
		f3d_vel_pair(t.x, t.y, t.z, s.a, s.b, vx, vy, vz);
		acc[0] += vx; acc[1] += vy; acc[2] += vz;
	}
	__device__ static void combine(const Tgt&, float (&)[NR]) {}
	__device__ static int slot(int c) { return c; }
	__device__ static void write(const Problem& p, const Consts&, int t, const double* s) {
		p.out[3 * size_t(t)] = float(s[0]);
		p.out[3 * size_t(t) + 1] = float(s[1]);
		p.out[3 * size_t(t) + 2] = float(s[2]);
	}
};
using F3DFew = FewForm2<F3DVelOp, 2, 4>;
constexpr int kF3DFewCfg = 5;   // the few-target form

// Velocity launch configurations: 0 scalar (1 target/thread, 128 threads),
// 1 scalar (4, 128), 2 packed (4, 128), 3 packed (2, 128), 4 packed (2, 256),
// 5 the few-target form. Default from GB300 timings (wake sheet, 20,000 and
// 100,000 points): 5 up to few_max_targets_vel2() targets, 0 below
// kSmallTargets, else 4; CVTX_GB300_F3D_CFG forces one.
int f3d_vel_cfg(int n_tgt, int n_fil) {
	static const int forced = [] {
		const char* e = std::getenv("CVTX_GB300_F3D_CFG");
		if (!e || !*e) return -1;
		const int c = std::atoi(e);
		return (c >= 0 && c <= kF3DFewCfg) ? c : -1;
	}();
	if (forced >= 0) return forced;
	if (n_tgt <= few_max_targets_vel2(n_fil)) return kF3DFewCfg;
	return n_tgt < kSmallTargets ? 0 : 4;
}
template <class F>
auto with_vel_cfg(int cfg, F&& f) {
	switch (cfg) {
	case 0: return f(std::integral_constant<int, 1>{}, std::integral_constant<int, 128>{}, std::false_type{});
	case 1: return f(std::integral_constant<int, 4>{}, std::integral_constant<int, 128>{}, std::false_type{});
	case 2: return f(std::integral_constant<int, 4>{}, std::integral_constant<int, 128>{}, std::true_type{});
	case 3: return f(std::integral_constant<int, 2>{}, std::integral_constant<int, 128>{}, std::true_type{});
	default: return f(std::integral_constant<int, 2>{}, std::integral_constant<int, 256>{}, std::true_type{});
	}
}

size_t f3d_vel_ws_bytes(int n_fil, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	if (f3d_vel_cfg(n_tgt, n_fil) == kF3DFewCfg)
		return F3DFew::plan(n_fil, n_tgt, num_sms, -1).ws_bytes;
	return with_vel_cfg(f3d_vel_cfg(n_tgt, n_fil), [&](auto t, auto n, auto pk) {
		return plan_vel<decltype(t)::value, decltype(n)::value, decltype(pk)::value>(
			n_fil, n_tgt, num_sms).ws_bytes;
	});
}
cudaError_t f3d_vel(const F3DVelProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	if (f3d_vel_cfg(p.n_tgt, p.n_fil) == kF3DFewCfg) {
		const Plan pl = F3DFew::plan(p.n_fil, p.n_tgt, env.num_sms,
			env.cap_to_ws ? split_cap_for(env.ws_bytes, 3, p.n_tgt) : -1);
		return F3DFew::launch(pl, p, F3DVelOp::Consts{0}, p.n_fil, p.n_tgt, env);
	}
	return with_vel_cfg(f3d_vel_cfg(p.n_tgt, p.n_fil), [&](auto t, auto n, auto pk) {
		return launch_vel<decltype(t)::value, decltype(n)::value, decltype(pk)::value>(p, env);
	});
}

// The F3D stretching pair as an operation of the few-target form: the same
// per-pair arithmetic as f3d_dvort_kernel (f3d_dvort_pair), 1/(4 pi) applied
// once per target.
struct F3DDvortOp {
	using Problem = F3DDvortProblem;
	struct Consts { int unused; };
	static constexpr int NC = 3, NR = 3;
	struct Tgt { float x, y, z, wx, wy, wz; };
	struct Src { float4 a, b; };
	__device__ static int n_src(const Problem& p) { return p.n_fil; }
	__device__ static int n_tgt(const Problem& p) { return p.n_tgt; }
	__device__ static Tgt target(const Problem& p, int t) {
		const float4 q = p.tgt[size_t(t) * p.tstride];
		const float4 w = p.tgt[size_t(t) * p.tstride + 1];
		return Tgt{q.x, q.y, q.z, w.x, w.y, w.z};
	}
	__device__ static Src source(const Problem& p, long long s) {
		return Src{p.fil[2 * s], p.fil[2 * s + 1]};
	}
	__device__ static void pair(const Consts&, const Tgt& t, const Src& s, float (&acc)[NR]) {
		float vx, vy, vz;
		f3d_dvort_pair(t.x, t.y, t.z, t.wx, t.wy, t.wz, s.a, s.b, vx, vy, vz);
		acc[0] += vx; acc[1] += vy; acc[2] += vz;
	}
	__device__ static void combine(const Tgt&, float (&)[NR]) {}
	__device__ static int slot(int c) { return c; }
	__device__ static void write(const Problem& p, const Consts&, int t, const double* s) {
		p.out[3 * size_t(t)] = float(kInv4Pi * s[0]);
		p.out[3 * size_t(t) + 1] = float(kInv4Pi * s[1]);
		p.out[3 * size_t(t) + 2] = float(kInv4Pi * s[2]);
	}
};
using F3DDvortFew = FewForm2<F3DDvortOp, 2, 4>;
constexpr int kF3DDvortFewCfg = 4;   // the few-target form

// Stretching launch configurations: 0 scalar (1 target/thread, 128
// threads), 1 packed (2, 128), 2 packed (4, 128), 3 packed (2, 256), 4 the
// few-target form. Default from GB300 timings (wake sheet of 20,000 to
// 1,000,000 filaments): 4 up to 512 targets (64 x 100,000: 41 us against
// 248 us for 0 or 1; 1,024 x 100,000: 351 against 304 us for 1), 1 below
// kSmallTargets (4,096 x 100,000: 787 us, against 1,295 us for 0), else 2
// (100,000 x 100,000: 16.8 ms, against 17.3 ms for 1 and 17.5 ms for 3).
// CVTX_GB300_F3D_DVORT_CFG forces one; CVTX_GB300_FEW_MAX moves the first
// threshold.
int f3d_dvort_cfg(int n_tgt, int) {
	static const int forced = [] {
		const char* e = std::getenv("CVTX_GB300_F3D_DVORT_CFG");
		if (!e || !*e) return -1;
		const int c = std::atoi(e);
		return (c >= 0 && c <= kF3DDvortFewCfg) ? c : -1;
	}();
	if (forced >= 0) return forced;
	const int few_max = few_max_override() >= 0 ? few_max_override() : 512;
	if (n_tgt <= few_max) return kF3DDvortFewCfg;
	return n_tgt < kSmallTargets ? 1 : 2;
}
template <class F>
auto with_dvort_cfg(int cfg, F&& f) {
	switch (cfg) {
	case 0: return f(std::integral_constant<int, 1>{}, std::integral_constant<int, 128>{}, std::false_type{});
	case 2: return f(std::integral_constant<int, 4>{}, std::integral_constant<int, 128>{}, std::true_type{});
	case 3: return f(std::integral_constant<int, 2>{}, std::integral_constant<int, 256>{}, std::true_type{});
	default: return f(std::integral_constant<int, 2>{}, std::integral_constant<int, 128>{}, std::true_type{});
	}
}

size_t f3d_dvort_ws_bytes(int n_fil, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	const int cfg = f3d_dvort_cfg(n_tgt, n_fil);
	if (cfg == kF3DDvortFewCfg) return F3DDvortFew::plan(n_fil, n_tgt, num_sms, -1).ws_bytes;
	return with_dvort_cfg(cfg, [&](auto t, auto n, auto pk) {
		return plan_dvort<decltype(t)::value, decltype(n)::value, decltype(pk)::value>(
			n_fil, n_tgt, num_sms).ws_bytes;
	});
}
cudaError_t f3d_dvort(const F3DDvortProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	const int cfg = f3d_dvort_cfg(p.n_tgt, p.n_fil);
	if (cfg == kF3DDvortFewCfg) {
		const Plan pl = F3DDvortFew::plan(p.n_fil, p.n_tgt, env.num_sms,
			env.cap_to_ws ? split_cap_for(env.ws_bytes, 3, p.n_tgt) : -1);
		return F3DDvortFew::launch(pl, p, F3DDvortOp::Consts{0}, p.n_fil, p.n_tgt, env);
	}
	return with_dvort_cfg(cfg, [&](auto t, auto n, auto pk) {
		return launch_dvort<decltype(t)::value, decltype(n)::value, decltype(pk)::value>(p, env);
	});
}
namespace {

// Influence-matrix configurations (point pairs per thread, unroll):
// 0 (4, 1), 1 (16, 1), 2 (16, 2), 3 (64, 1), 4 (64, 2), 5 (32, 2).
// CVTX_GB300_INF_CFG forces one. Default: of 0, 1 and 3, the one with the
// least (time per entry) / (fill of the last wave of CTAs); the time per
// entry of each, relative to 1, is from GB300 timings (25,000 x 20,000:
// 1.019 / 0.794 / 0.756 ms), where longer-lived CTAs amortise the filament
// tile load.
template <int PAIRS, int UNROLL>
int inf_resident_ctas() {
	static const int occ = resident_ctas(f3d_inf2_kernel<PAIRS, UNROLL>, kInfThreads, 0);
	return occ;
}

int inf_cfg(const F3DInfProblem& p, int num_sms) {
	static const int forced = [] {
		const char* e = std::getenv("CVTX_GB300_INF_CFG");
		if (!e || !*e) return -1;
		const int c = std::atoi(e);
		return (c >= 0 && c <= 5) ? c : -1;
	}();
	if (forced >= 0) return forced;
	const double fil_tiles = double((p.n_fil + kInfFils - 1) / kInfFils);
	const int cfgs[3] = {0, 1, 3};
	const int rows[3] = {inf_rows<4>(), inf_rows<16>(), inf_rows<64>()};
	const int occ[3] = {inf_resident_ctas<4, 1>(), inf_resident_ctas<16, 1>(),
		inf_resident_ctas<64, 1>()};
	const double per_entry[3] = {1.284, 1.0, 0.953};
	int best = 1;
	double best_cost = 1e300;
	for (int c = 0; c < 3; ++c) {
		const double ctas = std::ceil(double(p.n_mes) / rows[c]) * fil_tiles;
		const double wave = double(num_sms) * (occ[c] > 0 ? occ[c] : 1);
		const double fill = ctas / (std::ceil(ctas / wave) * wave);
		const double cost = per_entry[c] / fill;
		if (cost < best_cost) { best_cost = cost; best = cfgs[c]; }
	}
	return best;
}

template <int PAIRS, int UNROLL>
void launch_inf2(const F3DInfProblem& p, long long fil_tiles, cudaStream_t stream) {
	const long long row_tiles = (p.n_mes + inf_rows<PAIRS>() - 1) / inf_rows<PAIRS>();
	f3d_inf2_kernel<PAIRS, UNROLL><<<dim3(unsigned(row_tiles), unsigned(fil_tiles)),
		kInfThreads, 0, stream>>>(p);
}

}  // namespace

cudaError_t f3d_inf_mtrx(const F3DInfProblem& p, const LaunchEnv& env) {
	if (p.n_mes <= 0 || p.n_fil <= 0) return cudaSuccess;
	const long long fil_tiles = (p.n_fil + kInfFils - 1) / kInfFils;
	if (fil_tiles <= 65535) {
		switch (inf_cfg(p, env.num_sms)) {
		case 1: launch_inf2<16, 1>(p, fil_tiles, env.stream); break;
		case 2: launch_inf2<16, 2>(p, fil_tiles, env.stream); break;
		case 3: launch_inf2<64, 1>(p, fil_tiles, env.stream); break;
		case 4: launch_inf2<64, 2>(p, fil_tiles, env.stream); break;
		case 5: launch_inf2<32, 2>(p, fil_tiles, env.stream); break;
		default: launch_inf2<4, 1>(p, fil_tiles, env.stream); break;
		}
	} else {
		// more than 8.4M filaments: the grid-stride form
		const long long items = (long long)((p.n_fil + 3) / 4) * p.n_mes;
		const long long want = (items + 255) / 256;
		const int blocks = int(want < (long long)env.num_sms * 32 ? want : (long long)env.num_sms * 32);
		f3d_inf_kernel<<<blocks, 256, 0, env.stream>>>(p);
	}
	count_launch();
	return cudaGetLastError();
}

}  // namespace cvtx
