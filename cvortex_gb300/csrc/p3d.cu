// p3d.cu -- all-pairs 3D vortex particle kernels for sm_103a.
//
// Replaces the reference's OpenCL kernels cvtx_nb_P3D_{vel,dvort,visc_dvort,
// vort}_* (src/nbody.cl:38-197, 417-539) and their host code
// (src/ocl_P3D.cpp:150-899). Results follow the reference CPU path
// (src/P3D.cpp:51-144, 230-322): FP32 arithmetic per pair, coincident pairs
// contribute nothing, constant factors applied once per target.
//
// Kernel shape: one CTA owns TPT * NT targets (TPT per thread, registers)
// and streams a range of sources through shared memory in 256-record tiles
// (bulk copies, double-buffered). Each source is read once per thread with
// two broadcast 16-byte shared loads and reused for TPT targets. Tile partial
// sums (FP32) are folded into compensated (hi, lo) sums kept in shared
// memory. With one source split the CTA writes results directly; otherwise
// it writes FP64 partials that a finalize kernel combines in split order.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <mutex>
#include <type_traits>
#include "nbody.h"
#include "plan.cuh"
#include "regfuncs.cuh"
#include "p3d_induce.cuh"
#include "few.cuh"

namespace cvtx {

// Largest target count for the few-target form of the P3D velocity /
// stretching kernels, by source count (defined below).
int few_max_targets(int n_src);

RegConsts make_reg_consts_host(float sigma) {
	RegConsts c;
	const double s = sigma;
	const double as = std::fabs(s);
	c.inv_s = float(1.0 / as);
	c.inv_s2 = float(1.0 / (s * s));
	c.s2 = float(s * s);
	c.inv_s3 = float(1.0 / (as * as * as));
	const double rc = gaussian_rho_c();
	c.rho_c2 = float(rc * rc);
	c.exp2_half = float(-0.5 * 1.4426950408889634 / (s * s));
	return c;
}

namespace {

constexpr int kTile = kP3DTile;
using Stream2 = P3DStream;

RegConsts make_reg_consts(float sigma) { return make_reg_consts_host(sigma); }


}  // namespace

// Per-regularisation output scales (see regfuncs.cuh). Reference: vel uses
// 1/(4 pi) with rho = r/|sigma| (src/P3D.cpp:239,250); dvort uses the signed
// 1/(4 pi sigma^3) (src/P3D.cpp:102).
InduceConsts make_induce_consts(int reg, float sigma) {
	InduceConsts k;
	k.rc = make_reg_consts(sigma);
	const double inv4pi = 1.0 / (4.0 * 3.14159265358979323846);
	const double s = sigma;
	const double as = std::fabs(s);
	const double sgn = s < 0 ? -1.0 : 1.0;
	switch (reg) {
	case int(Reg::Singular):
	case int(Reg::Planetary):
		k.s_vel = -inv4pi;
		k.s_dv = sgn * inv4pi;
		k.k_scale = 3.0;
		break;
	case int(Reg::Winckelmans):  // rho-normalised G, K/3
		k.s_vel = -inv4pi / (as * as * as);
		k.s_dv = inv4pi / (s * s * s);
		k.k_scale = 3.0 / (s * s);
		break;
	default:  // Gaussian: rho-normalised G and K
		k.s_vel = -inv4pi / (as * as * as);
		k.s_dv = inv4pi / (s * s * s);
		k.k_scale = 1.0 / (s * s);
		break;
	}
	return k;
}

namespace {

// Sums per target (registers, FP32, reset every tile), as in
// p3d_induce.cuh: VEL u += G (d x alpha_s); DV A += G co, B += K (d.co) d with
// co = alpha_t x alpha_s rounded as the reference rounds it.
//
// One source-target pair in scalar FP32 into the register partials of one
// target. d = t - s; sv = source vorticity; a = alpha_t.
template <Reg R, bool VEL, bool DV, int NR>
__device__ __forceinline__ void induce_pair(float dx, float dy, float dz, const float4 sv,
	float ax, float ay, float az, const InduceConsts& kc, float (&acc)[NR])
{
	constexpr bool kFinite = FiniteAtZero<R>::value;
	const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
	// c = d x alpha_s
	const float cx = fmaf(dy, sv.z, -dz * sv.y);
	const float cy = fmaf(dz, sv.x, -dx * sv.z);
	const float cz = fmaf(dx, sv.y, -dy * sv.x);
	if (DV) {
		float G, K;
		RegP3D<R>::gk(r2, kc.rc, G, K);
		const bool nz = r2 > 0.f;
		G = nz ? G : 0.f;
		if (!kFinite) K = nz ? K : 0.f;
		constexpr int o = VEL ? 3 : 0;
		if (VEL) {
			acc[0] = fmaf(G, cx, acc[0]);
			acc[1] = fmaf(G, cy, acc[1]);
			acc[2] = fmaf(G, cz, acc[2]);
		}
		// co = alpha_t x alpha_s: two rounded products and their difference
		const float ox = __fsub_rn(__fmul_rn(ay, sv.z), __fmul_rn(az, sv.y));
		const float oy = __fsub_rn(__fmul_rn(az, sv.x), __fmul_rn(ax, sv.z));
		const float oz = __fsub_rn(__fmul_rn(ax, sv.y), __fmul_rn(ay, sv.x));
		acc[o + 0] = fmaf(G, ox, acc[o + 0]);
		acc[o + 1] = fmaf(G, oy, acc[o + 1]);
		acc[o + 2] = fmaf(G, oz, acc[o + 2]);
		const float pd = fmaf(dz, oz, fmaf(dy, oy, dx * ox));
		const float kk = K * pd;
		acc[o + 3] = fmaf(kk, dx, acc[o + 3]);
		acc[o + 4] = fmaf(kk, dy, acc[o + 4]);
		acc[o + 5] = fmaf(kk, dz, acc[o + 5]);
	} else {
		float G = RegP3D<R>::g(r2, kc.rc);
		if (!kFinite) G = r2 > 0.f ? G : 0.f;
		acc[0] = fmaf(G, cx, acc[0]);
		acc[1] = fmaf(G, cy, acc[1]);
		acc[2] = fmaf(G, cz, acc[2]);
	}
}

template <Reg R, bool VEL, bool DV, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_induce_kernel(const P3DInduceProblem p, const InduceConsts kc,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	constexpr int NC = (VEL ? 3 : 0) + (DV ? 6 : 0);     // compensated sums
	constexpr int NR = NC;                               // register partials
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;

	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;

	float tx[TPT], ty[TPT], tz[TPT], ax[TPT], ay[TPT], az[TPT];
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		int t = tbase + k * NT + tid;
		t = t < p.n_tgt ? t : p.n_tgt - 1;
		const float4 tp = p.tgt[size_t(t) * p.tstride];
		tx[k] = tp.x; ty[k] = tp.y; tz[k] = tp.z;
		if (DV) {
			const float4 tv = p.tgt[size_t(t) * p.tstride + 1];
			ax[k] = tv.x; ay[k] = tv.y; az[k] = tv.z;
		} else {
			ax[k] = ay[k] = az[k] = 0.f;
		}
	}
#pragma unroll
	for (int i = 0; i < NC * TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }

	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float acc[TPT][NR];
#pragma unroll
		for (int k = 0; k < TPT; ++k)
#pragma unroll
			for (int c = 0; c < NR; ++c) acc[k][c] = 0.f;

		auto body = [&](int j) {
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
#pragma unroll
			for (int k = 0; k < TPT; ++k)
				induce_pair<R, VEL, DV>(tx[k] - sp.x, ty[k] - sp.y, tz[k] - sp.z, sv,
					ax[k], ay[k], az[k], kc, acc[k]);
		};
		if (cnt == kTile) {
#pragma unroll 2
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int c = 0; c < NC; ++c) {
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const int i = (c * TPT + k) * NT + tid;
				float h = hi[i], l = lo[i];
				fold_twosum(h, l, acc[k][c]);
				hi[i] = h; lo[i] = l;
			}
		}
	};

	if (!Stream2::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;

#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
		double s[NC];
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			s[c] = double(hi[i]) + double(lo[i]);
		}
		if (gridDim.y == 1) {
			write_induce<VEL, DV>(p, kc, t, s);
		} else {
#pragma unroll
			for (int c = 0; c < NC; ++c)
				partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s[c];
		}
	}
}

// Packed variant of p3d_induce_kernel (two targets per f32x2 lane pair; see
// induce2_block in p3d_induce.cuh). CTA (x, y) = (target block, source split).
template <Reg R, bool VEL, bool DV, int TPT, int NT, int UNROLL, int TILE, int MINB>
__global__ void __launch_bounds__(NT, MINB)
p3d_induce2_kernel(const P3DInduceProblem p, const InduceConsts kc,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	constexpr int NC = InduceNC<VEL, DV>::value;
	extern __shared__ __align__(16) unsigned char smem[];
	if (!P3DStreamT<TILE>::init(smem, err)) return;
	unsigned tcount = 0;
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	induce2_block<R, VEL, DV, TPT, NT, UNROLL, TILE>(p, kc, blockIdx.x * (TPT * NT), s_begin, n_s,
		smem, err,
		tcount, [&](int t, const double* acc) {
			if (gridDim.y == 1) {
				write_induce<VEL, DV>(p, kc, t, acc);
			} else {
#pragma unroll
				for (int c = 0; c < NC; ++c)
					partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = acc[c];
			}
		});
}

template <bool VEL, bool DV>
__global__ void p3d_induce_finalize(const P3DInduceProblem p, const InduceConsts kc,
	const double* __restrict__ partial, int n_split)
{
	constexpr int NC = (VEL ? 3 : 0) + (DV ? 6 : 0);
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= p.n_tgt) return;
	double s[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) s[c] = 0.0;
	for (int sp = 0; sp < n_split; ++sp)
#pragma unroll
		for (int c = 0; c < NC; ++c) s[c] += partial[(size_t(sp) * NC + c) * p.n_tgt + t];
	write_induce<VEL, DV>(p, kc, t, s);
}

// The P3D velocity / stretching pair as an operation of the few-target form
// (few.cuh): the same per-pair arithmetic as p3d_induce_kernel.
template <Reg R, bool VEL, bool DV>
struct P3DInduceOp {
	using Problem = P3DInduceProblem;
	using Consts = InduceConsts;
	static constexpr int NC = InduceNC<VEL, DV>::value;
	static constexpr int NR = NC;
	struct Tgt { float x, y, z, ax, ay, az; };
	struct Src { float4 pos, vort; };
	__device__ static int n_src(const Problem& p) { return p.n_src; }
	__device__ static int n_tgt(const Problem& p) { return p.n_tgt; }
	__device__ static Tgt target(const Problem& p, int t) {
		const float4 tp = p.tgt[size_t(t) * p.tstride];
		Tgt g{tp.x, tp.y, tp.z, 0.f, 0.f, 0.f};
		if (DV) {
			const float4 tv = p.tgt[size_t(t) * p.tstride + 1];
			g.ax = tv.x; g.ay = tv.y; g.az = tv.z;
		}
		return g;
	}
	__device__ static Src source(const Problem& p, long long s) {
		return Src{p.src[2 * s], p.src[2 * s + 1]};
	}
	__device__ static void pair(const Consts& k, const Tgt& t, const Src& s, float (&acc)[NR]) {
		induce_pair<R, VEL, DV>(t.x - s.pos.x, t.y - s.pos.y, t.z - s.pos.z, s.vort,
			t.ax, t.ay, t.az, k, acc);
	}
	__device__ static void combine(const Tgt&, float (&)[NR]) {}
	__device__ static int slot(int c) { return c; }
	__device__ static void write(const Problem& p, const Consts& k, int t, const double* s) {
		write_induce<VEL, DV>(p, k, t, s);
	}
};

// ---------------------------------------------------------------------------
// Viscous vorticity exchange (PSE), reference src/P3D.cpp:116-144:
//   out_t = (2 nu / sigma^2) sum_s (alpha_s V_t - alpha_t V_s) eta(rho)
// ---------------------------------------------------------------------------
struct ViscConsts { RegConsts rc; double scale; };

template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_visc_kernel(const P3DViscProblem p, const ViscConsts vc,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	constexpr int NC = 3;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;

	float tx[TPT], ty[TPT], tz[TPT], tv_[TPT], ax[TPT], ay[TPT], az[TPT];
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		int t = tbase + k * NT + tid;
		t = t < p.n_tgt ? t : p.n_tgt - 1;
		const float4 tp = p.tgt[size_t(t) * p.tstride];
		const float4 tw = p.tgt[size_t(t) * p.tstride + 1];
		tx[k] = tp.x; ty[k] = tp.y; tz[k] = tp.z; tv_[k] = tp.w;
		ax[k] = tw.x; ay[k] = tw.y; az[k] = tw.z;
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
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const float dx = sp.x - tx[k];
				const float dy = sp.y - ty[k];
				const float dz = sp.z - tz[k];
				const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
				float e = RegP3D<R>::eta(r2, vc.rc);
				e = r2 > 0.f ? e : 0.f;
				// alpha_s V_t - alpha_t V_s, as the reference forms it per pair
				const float wx = fmaf(sv.x, tv_[k], -ax[k] * sp.w);
				const float wy = fmaf(sv.y, tv_[k], -ay[k] * sp.w);
				const float wz = fmaf(sv.z, tv_[k], -az[k] * sp.w);
				acc[0][k] = fmaf(e, wx, acc[0][k]);
				acc[1][k] = fmaf(e, wy, acc[1][k]);
				acc[2][k] = fmaf(e, wz, acc[2][k]);
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
	if (!Stream2::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;

#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(vc.scale * s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

// Packed variant (two targets per f32x2 lane pair).
template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_visc2_kernel(const P3DViscProblem p, const ViscConsts vc,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int NC = 3, H = TPT / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float2 tx[H], ty[H], tz[H], tv[H], nax[H], nay[H], naz[H];
#pragma unroll
	for (int h = 0; h < H; ++h) {
		float4 q[2], w[2];
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			int t = tbase + (2 * h + e) * NT + tid;
			t = t < p.n_tgt ? t : p.n_tgt - 1;
			q[e] = p.tgt[size_t(t) * p.tstride];
			w[e] = p.tgt[size_t(t) * p.tstride + 1];
		}
		tx[h] = make_float2(q[0].x, q[1].x); ty[h] = make_float2(q[0].y, q[1].y);
		tz[h] = make_float2(q[0].z, q[1].z); tv[h] = make_float2(q[0].w, q[1].w);
		nax[h] = make_float2(-w[0].x, -w[1].x); nay[h] = make_float2(-w[0].y, -w[1].y);
		naz[h] = make_float2(-w[0].z, -w[1].z);
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
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
			const float2 sx = bc2(sp.x), sy = bc2(sp.y), sz = bc2(sp.z), vs = bc2(sp.w);
#pragma unroll
			for (int h = 0; h < H; ++h) {
				const float2 dx = __fadd2_rn(sx, make_float2(-tx[h].x, -tx[h].y));
				const float2 dy = __fadd2_rn(sy, make_float2(-ty[h].x, -ty[h].y));
				const float2 dz = __fadd2_rn(sz, make_float2(-tz[h].x, -tz[h].y));
				const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
				float2 e = RegEta2<R>::eta2(r2, vc.rc);
				e.x = r2.x > 0.f ? e.x : 0.f;
				e.y = r2.y > 0.f ? e.y : 0.f;
				// alpha_s V_t - alpha_t V_s
				const float2 wx = __ffma2_rn(bc2(sv.x), tv[h], __fmul2_rn(nax[h], vs));
				const float2 wy = __ffma2_rn(bc2(sv.y), tv[h], __fmul2_rn(nay[h], vs));
				const float2 wz = __ffma2_rn(bc2(sv.z), tv[h], __fmul2_rn(naz[h], vs));
				acc[0][h] = __ffma2_rn(e, wx, acc[0][h]);
				acc[1][h] = __ffma2_rn(e, wy, acc[1][h]);
				acc[2][h] = __ffma2_rn(e, wz, acc[2][h]);
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
	if (!Stream2::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(vc.scale * s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

__global__ void p3_finalize_scaled(float* __restrict__ out, int n_tgt,
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

// ---------------------------------------------------------------------------
// Vorticity field with the reference CPU's 5 sigma box cut-off
// (src/P3D.cpp:298-322): out = sum_{|dx|,|dy|,|dz| < 5 sigma} zeta(rho) alpha_s
// / (4 pi sigma^3).
// ---------------------------------------------------------------------------
// (singular: zeta = 0, so its field is a memset and needs no kernel)
template <Reg R> struct ZetaP3D;
template <> struct ZetaP3D<Reg::Winckelmans> {
	__device__ __forceinline__ static float z(float r2, const RegConsts& c) {
		const float q = fmaf(r2, c.inv_s2, 1.f);
		const float s = rsqrt_approx(q);
		const float s2 = s * s;
		return 7.5f * (s2 * s2 * s2 * s);
	} };
template <> struct ZetaP3D<Reg::Planetary> {
	__device__ __forceinline__ static float z(float r2, const RegConsts& c) {
		return r2 < c.s2 ? 3.f : 0.f; } };
template <> struct ZetaP3D<Reg::Gaussian> {
	__device__ __forceinline__ static float z(float r2, const RegConsts& c) {
		return kSqrt2OverPi * exp2f(r2 * c.exp2_half); } };

template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_vort_kernel(const P3DVortProblem p, const RegConsts rc, float cutoff,
	double scale, double* __restrict__ partial, int src_per_split, unsigned* err)
{
	constexpr int NC = 3;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
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
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const float dx = sp.x - tx[k];
				const float dy = sp.y - ty[k];
				const float dz = sp.z - tz[k];
				// the box test as one three-input max: NaN in any component
				// gives NaN, which fails it, as each separate test would
				const bool in = max3_nan(fabsf(dx), fabsf(dy), fabsf(dz)) < cutoff;
				const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
				float z = ZetaP3D<R>::z(r2, rc);
				z = in ? z : 0.f;
				acc[0][k] = fmaf(z, sv.x, acc[0][k]);
				acc[1][k] = fmaf(z, sv.y, acc[1][k]);
				acc[2][k] = fmaf(z, sv.z, acc[2][k]);
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
	if (!Stream2::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(scale * s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

// Packed form (two targets per f32x2 lane pair); zeta's shape is
// ZetaShape2 (p3d_induce.cuh), its constant factor in the FP64 output scale.
template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_vort2_kernel(const P3DVortProblem p, const RegConsts rc, float cutoff,
	double scale, double* __restrict__ partial, int src_per_split, unsigned* err)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int NC = 3, H = TPT / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float2 ntx[H], nty[H], ntz[H];   // negated target coordinates
#pragma unroll
	for (int h = 0; h < H; ++h) {
		float4 q[2];
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			int t = tbase + (2 * h + e) * NT + tid;
			t = t < p.n_tgt ? t : p.n_tgt - 1;
			q[e] = p.tgt[size_t(t) * p.tstride];
		}
		ntx[h] = make_float2(-q[0].x, -q[1].x);
		nty[h] = make_float2(-q[0].y, -q[1].y);
		ntz[h] = make_float2(-q[0].z, -q[1].z);
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
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
			const float2 sx = bc2(sp.x), sy = bc2(sp.y), sz = bc2(sp.z);
#pragma unroll
			for (int h = 0; h < H; ++h) {
				// source - target, rounded once as in the scalar form
				const float2 dx = __fadd2_rn(sx, ntx[h]);
				const float2 dy = __fadd2_rn(sy, nty[h]);
				const float2 dz = __fadd2_rn(sz, ntz[h]);
				const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
				float2 z = ZetaShape2<R>::z(r2, rc);
				const bool in0 = max3_nan(fabsf(dx.x), fabsf(dy.x), fabsf(dz.x)) < cutoff;
				const bool in1 = max3_nan(fabsf(dx.y), fabsf(dy.y), fabsf(dz.y)) < cutoff;
				z.x = in0 ? z.x : 0.f;
				z.y = in1 ? z.y : 0.f;
				acc[0][h] = __ffma2_rn(z, bc2(sv.x), acc[0][h]);
				acc[1][h] = __ffma2_rn(z, bc2(sv.y), acc[1][h]);
				acc[2][h] = __ffma2_rn(z, bc2(sv.z), acc[2][h]);
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
	if (!Stream2::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[3 * size_t(t) + c] = float(scale * s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <int TPT, int NT, int NC>
constexpr size_t smem_bytes() {
	return Stream2::kSmemBytes + size_t(2) * NC * TPT * NT * sizeof(float);
}

// ---- induce launch configurations ------------------------------------------
// A configuration is (targets per thread, threads per CTA, packed f32x2 or
// scalar arithmetic). The table below is what the autotuner chooses from;
// without a tuned entry, up to few_max_targets() targets use configuration 10
// (p3d_induce_few_kernel: sources spread over the threads), fewer than
// kSmallTargets configuration 0 (one target per thread, so the source
// dimension can be split across more CTAs) and larger problems the measured
// per-(regularisation, ops) choice of kMidCfg / kLargeCfg below.
constexpr int kSmallTargets = 8192;
constexpr int kFewCfg = 10;

struct CfgSpec { int tpt, nt; bool packed; };
constexpr CfgSpec kCfg[] = {
	{1, 128, false}, {4, 128, false}, {4, 128, true}, {2, 128, true},
	{4, 64, true},   {2, 256, true},  {6, 64, true},  {4, 128, true},
	{4, 128, true},  {2, 128, true},  {4, 256, false},   // 10: few targets (TT = 4 or 8)
};
// Configurations 7-9 repeat shapes with another source-loop unroll factor
// (7: 1, 8 and 9: 4; all others 2). (Also timed on a GB300 and left out:
// five resident CTAs per SM with 96-source tiles, which spilled registers and
// ran 20-30 % slower, and 6 x 128 / 8 x 64 blocking, within 2 % of these.)
constexpr int kNumCfg = int(sizeof(kCfg) / sizeof(kCfg[0]));

template <Reg R, bool VEL, bool DV, int TPT, int NT, bool PK, int UNROLL = 2,
	int TILE = kTile, int MINB = 1>
struct InduceVariant {
	static constexpr int NC = (VEL ? 3 : 0) + (DV ? 6 : 0);
	static constexpr size_t kSmem = PK ? induce_smem_bytes<TPT, NT, NC, TILE>()
	                                   : smem_bytes<TPT, NT, NC>();
	using Fn = void (*)(const P3DInduceProblem, const InduceConsts, double*, int, unsigned*);
	static Fn fn() {
		if constexpr (PK) return p3d_induce2_kernel<R, VEL, DV, TPT, NT, UNROLL, TILE, MINB>;
		else return p3d_induce_kernel<R, VEL, DV, TPT, NT>;
	}
	static int occupancy() {
		static const int occ = resident_ctas(fn(), NT, kSmem);
		return occ;
	}
	// max_split < 0: this kernel's own cap (64 splits)
	static Plan plan(int n_src, int n_tgt, int num_sms, int max_split, int min_split = 1) {
		return make_plan(n_src, n_tgt, TPT * NT, PK ? TILE : kTile, NC, num_sms * occupancy(), kSmem,
			max_split < 0 ? 64 : max_split, min_split);
	}
	static cudaError_t launch(const Plan& pl, const P3DInduceProblem& p, const LaunchEnv& env) {
		if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
		const InduceConsts kc = make_induce_consts(int(R), p.sigma);
		double* partial = static_cast<double*>(env.ws);
		fn()<<<dim3(pl.n_tblocks, pl.n_split), NT, pl.smem, env.stream>>>(
			p, kc, partial, pl.src_per_split, env.err);
		count_launch();
		if (pl.n_split > 1) {
			p3d_induce_finalize<VEL, DV><<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
				p, kc, partial, pl.n_split);
			count_launch();
		}
		return cudaGetLastError();
	}
};

// The few-target form (few.cuh) as configuration 10: Plan.n_tblocks =
// target groups, n_split = source chunks, src_per_split = chunk length.
// Targets per CTA (few.cuh, FewForm2): 4 / 8 for vel, 2 / 4 for stretching.
template <Reg R, bool VEL, bool DV>
struct FewVariant {
	static constexpr int NC = InduceNC<VEL, DV>::value;
	using Form = FewForm2<P3DInduceOp<R, VEL, DV>, (VEL && !DV) ? 4 : 2, (VEL && !DV) ? 8 : 4>;
	static Plan plan(int n_src, int n_tgt, int num_sms, int max_split, int = 1) {
		return Form::plan(n_src, n_tgt, num_sms, max_split);
	}
	static cudaError_t launch(const Plan& pl, const P3DInduceProblem& p, const LaunchEnv& env) {
		return Form::launch(pl, p, make_induce_consts(int(R), p.sigma), p.n_src, p.n_tgt, env);
	}
};

template <Reg R, bool VEL, bool DV, class F>
auto with_cfg(int ci, F&& f) {
	switch (ci) {
	case 0: return f(InduceVariant<R, VEL, DV, 1, 128, false>{});
	case 1: return f(InduceVariant<R, VEL, DV, 4, 128, false>{});
	case 2: return f(InduceVariant<R, VEL, DV, 4, 128, true>{});
	case 3: return f(InduceVariant<R, VEL, DV, 2, 128, true>{});
	case 4: return f(InduceVariant<R, VEL, DV, 4, 64, true>{});
	case 5: return f(InduceVariant<R, VEL, DV, 2, 256, true>{});
	case 6: return f(InduceVariant<R, VEL, DV, 6, 64, true>{});
	case 7: return f(InduceVariant<R, VEL, DV, 4, 128, true, 1>{});
	case 8: return f(InduceVariant<R, VEL, DV, 4, 128, true, 4>{});
	case 9: return f(InduceVariant<R, VEL, DV, 2, 128, true, 4>{});
	default: return f(FewVariant<R, VEL, DV>{});
	}
}

template <class F>
auto with_reg_ops(int reg, unsigned ops, F&& f) {
	auto by_ops = [&](auto rtag) {
		constexpr Reg R = decltype(rtag)::value;
		switch (ops) {
		case kOpVel: return f(std::integral_constant<Reg, R>{}, std::true_type{}, std::false_type{});
		case kOpDvort: return f(std::integral_constant<Reg, R>{}, std::false_type{}, std::true_type{});
		default: return f(std::integral_constant<Reg, R>{}, std::true_type{}, std::true_type{});
		}
	};
	switch (reg) {
	case 0: return by_ops(std::integral_constant<Reg, Reg::Singular>{});
	case 1: return by_ops(std::integral_constant<Reg, Reg::Winckelmans>{});
	case 2: return by_ops(std::integral_constant<Reg, Reg::Planetary>{});
	default: return by_ops(std::integral_constant<Reg, Reg::Gaussian>{});
	}
}

// Tuned configuration per (regularisation, ops, size bucket); -1 = default.
std::atomic<int> g_tuned[4][4][kNumSizeBuckets];
const bool g_tuned_init = [] {
	for (auto& a : g_tuned) for (auto& b : a) for (auto& c : b) c.store(-1);
	return true;
}();

int env_cfg() {
	static const int v = [] {
		const char* e = std::getenv("CVTX_GB300_P3D_CFG");
		if (!e || !*e) return -1;
		const int c = std::atoi(e);
		return (c >= 0 && c < kNumCfg) ? c : -1;
	}();
	return v;
}

// Built-in choice per (regularisation, ops) for 8,192-32,767 targets and for
// 32,768 or more, from timings of every configuration on a GB300 (vortex
// ring, sigma 0.05; 20,000 and 100,000 / 400,000 targets). Below 8,192
// targets configuration 0 was fastest for every regularisation and op.
// Index: [reg: singular, winckelmans, planetary, gaussian][ops: -, vel, dvort, both].
constexpr signed char kMidCfg[4][4] = {
	{2, 3, 5, 3}, {2, 3, 0, 2}, {2, 3, 0, 2}, {2, 6, 5, 3}};
constexpr signed char kLargeCfg[4][4] = {
	{2, 3, 5, 3}, {2, 6, 6, 2}, {2, 4, 2, 2}, {2, 6, 4, 9}};

int choose_cfg(int reg, unsigned ops, int n_tgt, int n_src) {
	const int forced = env_cfg();
	if (forced >= 0) return forced;
	const int t = g_tuned[reg & 3][ops & 3][size_bucket(n_tgt)].load(std::memory_order_relaxed);
	if (t >= 0 && t < kNumCfg) return t;
	if (n_tgt <= few_max_targets(n_src)) return kFewCfg;
	if (n_tgt < kSmallTargets) return 0;
	return n_tgt < 32768 ? kMidCfg[reg & 3][ops & 3] : kLargeCfg[reg & 3][ops & 3];
}

size_t induce_ws(int reg, unsigned ops, int n_src, int n_tgt, int num_sms, int cfg) {
	return with_reg_ops(reg, ops, [&](auto rt, auto vt, auto dt) {
		constexpr Reg R = decltype(rt)::value;
		constexpr bool VEL = decltype(vt)::value, DV = decltype(dt)::value;
		return with_cfg<R, VEL, DV>(cfg, [&](auto var) {
			return decltype(var)::plan(n_src, n_tgt, num_sms, -1).ws_bytes;
		});
	});
}

cudaError_t induce_launch(int reg, unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env,
	int cfg, bool bounded) {
	return with_reg_ops(reg, ops, [&](auto rt, auto vt, auto dt) {
		constexpr Reg R = decltype(rt)::value;
		constexpr bool VEL = decltype(vt)::value, DV = decltype(dt)::value;
		return with_cfg<R, VEL, DV>(cfg, [&](auto var) {
			using V = decltype(var);
			// capped: the FP64 split partials must fit env.ws_bytes
			const int max_split = (bounded || env.cap_to_ws)
				? split_cap_for(env.ws_bytes, V::NC, p.n_tgt) : -1;
			return V::launch(V::plan(p.n_src, p.n_tgt, env.num_sms, max_split,
				min_split_for(env, p.n_src)), p, env);
		});
	});
}

template <Reg R, int TPT, int NT, bool PK>
auto visc_kernel() {
	if constexpr (PK) return p3d_visc2_kernel<R, TPT, NT>;
	else return p3d_visc_kernel<R, TPT, NT>;
}

template <Reg R, int TPT, int NT, bool PK>
Plan plan_visc(int n_src, int n_tgt, int num_sms, int max_split = 64) {
	constexpr size_t smem = smem_bytes<TPT, NT, 3>();
	static const int occ = resident_ctas(visc_kernel<R, TPT, NT, PK>(), NT, smem);
	return make_plan(n_src, n_tgt, TPT * NT, kTile, 3, num_sms * occ, smem, max_split);
}

template <Reg R, int TPT, int NT, bool PK>
cudaError_t launch_visc(const P3DViscProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_visc<R, TPT, NT, PK>(p.n_src, p.n_tgt, env.num_sms,
		env.cap_to_ws ? split_cap_for(env.ws_bytes, 3, p.n_tgt) : 64);
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	ViscConsts vc;
	vc.rc = make_reg_consts(p.sigma);
	const double base = 2.0 * double(p.nu) / (double(p.sigma) * double(p.sigma));
	vc.scale = base * (R == Reg::Winckelmans ? 52.5 : double(kSqrt2OverPi));
	double* partial = static_cast<double*>(env.ws);
	dim3 grid(pl.n_tblocks, pl.n_split);
	visc_kernel<R, TPT, NT, PK>()<<<grid, NT, pl.smem, env.stream>>>(
		p, vc, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		p3_finalize_scaled<<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
			p.out, p.n_tgt, partial, pl.n_split, vc.scale);
		count_launch();
	}
	return cudaGetLastError();
}

template <Reg R_, int TPT_, bool PK_> struct vort_tag {
	static constexpr Reg R = R_;
	static constexpr int TPT = TPT_;
	static constexpr bool PK = PK_;
};

template <Reg R, int TPT, int NT, bool PK>
auto vort_kernel() {
	if constexpr (PK) return p3d_vort2_kernel<R, TPT, NT>;
	else return p3d_vort_kernel<R, TPT, NT>;
}

template <Reg R, int TPT, int NT, bool PK>
Plan plan_vort(int n_src, int n_tgt, int num_sms, int max_split = 64) {
	constexpr size_t smem = smem_bytes<TPT, NT, 3>();
	static const int occ = resident_ctas(vort_kernel<R, TPT, NT, PK>(), NT, smem);
	return make_plan(n_src, n_tgt, TPT * NT, kTile, 3, num_sms * occ, smem, max_split);
}

template <Reg R, int TPT, int NT, bool PK>
cudaError_t launch_vort(const P3DVortProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_vort<R, TPT, NT, PK>(p.n_src, p.n_tgt, env.num_sms,
		env.cap_to_ws ? split_cap_for(env.ws_bytes, 3, p.n_tgt) : 64);
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	const RegConsts rc = make_reg_consts(p.sigma);
	const double s = p.sigma;
	double scale = 1.0 / (4.0 * 3.14159265358979323846 * s * s * s);
	if constexpr (PK) scale *= ZetaShape2<R>::kFactor;
	const float cutoff = 5.f * p.sigma;
	double* partial = static_cast<double*>(env.ws);
	dim3 grid(pl.n_tblocks, pl.n_split);
	vort_kernel<R, TPT, NT, PK>()<<<grid, NT, pl.smem, env.stream>>>(
		p, rc, cutoff, scale, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		p3_finalize_scaled<<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
			p.out, p.n_tgt, partial, pl.n_split, scale);
		count_launch();
	}
	return cudaGetLastError();
}

}  // namespace

// Largest target count for the few-target form, from GB300 timings against
// configuration 0 (vortex ring, vel and vel+dvort, 1 to 2,048 targets): it
// is faster up to 256 targets at 100,000 sources and up to 2,048 at
// 1,000,000, where the split form's 64-split cap leaves SMs idle.
// CVTX_GB300_FEW_MAX overrides it.
int few_max_override() {
	static const int forced = [] {
		const char* e = std::getenv("CVTX_GB300_FEW_MAX");
		return (e && *e) ? std::atoi(e) : -1;
	}();
	return forced;
}

int few_max_targets(int n_src) {
	const int forced = few_max_override();
	if (forced >= 0) return forced;
	return n_src >= 262144 ? 2048 : 256;
}

size_t p3d_induce_ws_bytes(int reg, unsigned ops, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	return induce_ws(reg, ops, n_src, n_tgt, num_sms, choose_cfg(reg, ops, n_tgt, n_src));
}

// The self-interaction form when it applies to the problem and the launch
// (no CTA lifetime cap, no forced or tuned configuration).
static bool use_self_form(int reg, unsigned ops, const P3DInduceProblem& p, int cta_src_cap) {
	if (cta_src_cap > 0 || env_cfg() >= 0) return false;
	if (g_tuned[reg & 3][ops & 3][size_bucket(p.n_tgt)].load(std::memory_order_relaxed) >= 0)
		return false;
	return p3d_self_form_applies(reg, ops, p);
}

size_t p3d_induce_ws_bytes_for(int reg, unsigned ops, const P3DInduceProblem& p, int num_sms) {
	if (p.n_tgt <= 0) return 0;
	const size_t base = p3d_induce_ws_bytes(reg, ops, p.n_src, p.n_tgt, num_sms);
	if (!use_self_form(reg, ops, p, 0)) return base;
	const size_t self = p3d_self_ws_bytes(reg, ops, p.n_tgt, num_sms);
	return self == SIZE_MAX ? base : std::max(base, self);
}

cudaError_t p3d_induce(int reg, unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	if (reg < 0 || reg > 3 || ops < 1 || ops > 3) return cudaErrorInvalidValue;
	if (use_self_form(reg, ops, p, env.cta_src_cap) &&
		p3d_self_ws_bytes(reg, ops, p.n_tgt, env.num_sms, env.cap_to_ws ? env.ws_bytes : 0) <=
			env.ws_bytes)
		return p3d_self(reg, ops, p, env);
	return induce_launch(reg, ops, p, env, choose_cfg(reg, ops, p.n_tgt, p.n_src), false);
}

cudaError_t p3d_induce_bounded(int reg, unsigned ops, const P3DInduceProblem& p,
	const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	if (reg < 0 || reg > 3 || ops < 1 || ops > 3) return cudaErrorInvalidValue;
	return induce_launch(reg, ops, p, env, choose_cfg(reg, ops, p.n_tgt, p.n_src), true);
}

int p3d_induce_num_configs() { return kNumCfg; }

bool p3d_induce_config(int cfg, int* tpt, int* nt, int* packed) {
	if (cfg < 0 || cfg >= kNumCfg) return false;
	*tpt = kCfg[cfg].tpt; *nt = kCfg[cfg].nt; *packed = kCfg[cfg].packed ? 1 : 0;
	return true;
}

bool p3d_induce_set_tuned(int reg, unsigned ops, int bucket, int cfg) {
	if (reg < 0 || reg > 3 || ops < 1 || ops > 3 || bucket < 0 || bucket >= kNumSizeBuckets ||
		cfg < -1 || cfg >= kNumCfg) return false;
	g_tuned[reg][ops][bucket].store(cfg);
	return true;
}

int p3d_induce_current_config(int reg, unsigned ops, int n_tgt) {
	return choose_cfg(reg & 3, ops & 3, n_tgt, 0);
}

size_t p3d_visc_ws_bytes(int reg, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	const bool small = n_tgt < kSmallTargets;
	if (reg == int(Reg::Winckelmans))
		return small ? plan_visc<Reg::Winckelmans, 1, 128, false>(n_src, n_tgt, num_sms).ws_bytes
		             : plan_visc<Reg::Winckelmans, 4, 128, true>(n_src, n_tgt, num_sms).ws_bytes;
	if (reg == int(Reg::Gaussian))
		return small ? plan_visc<Reg::Gaussian, 1, 128, false>(n_src, n_tgt, num_sms).ws_bytes
		             : plan_visc<Reg::Gaussian, 4, 128, true>(n_src, n_tgt, num_sms).ws_bytes;
	return 0;
}

// Only Winckelmans and Gaussian have an eta function; the runtime handles the
// other regularisations (zeros and a warning) without launching anything.
size_t p3d_visc_ws_bytes_for(int reg, const P3DViscProblem& p, int num_sms) {
	if (p.n_tgt <= 0) return 0;
	const size_t base = p3d_visc_ws_bytes(reg, p.n_src, p.n_tgt, num_sms);
	if (!p3d_visc_self_form_applies(reg, p)) return base;
	const size_t self = p3d_visc_self_ws_bytes(reg, p.n_tgt, num_sms);
	return self == SIZE_MAX ? base : std::max(base, self);
}

cudaError_t p3d_visc(int reg, const P3DViscProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	if (env.cta_src_cap == 0 && p3d_visc_self_form_applies(reg, p) &&
		p3d_visc_self_ws_bytes(reg, p.n_tgt, env.num_sms, env.cap_to_ws ? env.ws_bytes : 0) <=
			env.ws_bytes)
		return p3d_visc_self(reg, p, env);
	const bool small = p.n_tgt < kSmallTargets;
	if (reg == int(Reg::Winckelmans))
		return small ? launch_visc<Reg::Winckelmans, 1, 128, false>(p, env)
		             : launch_visc<Reg::Winckelmans, 4, 128, true>(p, env);
	if (reg == int(Reg::Gaussian))
		return small ? launch_visc<Reg::Gaussian, 1, 128, false>(p, env)
		             : launch_visc<Reg::Gaussian, 4, 128, true>(p, env);
	return cudaErrorInvalidValue;
}

// Vorticity-field configurations (targets per thread, 128 threads per CTA):
// 0 scalar (4), 1 packed (4), 2 packed (8), 3 packed (2). Default from GB300
// timings (vortex ring, 20,000 / 100,000 / 400,000 targets): 0 below
// kSmallTargets targets, 3 up to 65,535, else 2; CVTX_GB300_VORT_CFG forces
// one.
// The singular regularisation's zeta is identically zero (reference
// src/VortFunc.cpp:68-70), so its field is zero without evaluating any pair.
int vort_forced_cfg() {
	static const int forced = [] {
		const char* e = std::getenv("CVTX_GB300_VORT_CFG");
		if (!e || !*e) return -1;
		const int c = std::atoi(e);
		return (c >= 0 && c <= 3) ? c : -1;
	}();
	return forced;
}
int vort_cfg(int n_tgt) {
	const int forced = vort_forced_cfg();
	if (forced >= 0) return forced;
	return n_tgt < kSmallTargets ? 0 : n_tgt < 65536 ? 3 : 2;
}

template <Reg R, typename F>
cudaError_t with_vort_tpt(int cfg, F&& f) {
	switch (cfg) {
	case 0: return f(vort_tag<R, 4, false>{});
	case 2: return f(vort_tag<R, 8, true>{});
	case 3: return f(vort_tag<R, 2, true>{});
	default: return f(vort_tag<R, 4, true>{});
	}
}

template <typename F>
cudaError_t with_vort_cfg(int reg, int n_tgt, F&& f) {
	const int cfg = vort_cfg(n_tgt);
	switch (reg) {
	case 1: return with_vort_tpt<Reg::Winckelmans>(cfg, f);
	case 2: return with_vort_tpt<Reg::Planetary>(cfg, f);
	case 3: return with_vort_tpt<Reg::Gaussian>(cfg, f);
	default: return cudaErrorInvalidValue;
	}
}

size_t p3d_vort_ws_bytes(int reg, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0 || reg == int(Reg::Singular)) return 0;
	size_t ws = 0;
	with_vort_cfg(reg, n_tgt, [&](auto tag) {
		using T = decltype(tag);
		ws = plan_vort<T::R, T::TPT, 128, T::PK>(n_src, n_tgt, num_sms).ws_bytes;
		return cudaSuccess;
	});
	return ws;
}

static bool use_vort_self(int reg, const P3DVortProblem& p, int cta_src_cap) {
	return cta_src_cap == 0 && vort_forced_cfg() < 0 && p3d_vort_self_form_applies(reg, p);
}

size_t p3d_vort_ws_bytes_for(int reg, const P3DVortProblem& p, int num_sms) {
	const size_t base = p3d_vort_ws_bytes(reg, p.n_src, p.n_tgt, num_sms);
	if (p.n_tgt <= 0 || !use_vort_self(reg, p, 0)) return base;
	const size_t self = p3d_vort_self_ws_bytes(reg, p.n_tgt, num_sms);
	return self == SIZE_MAX ? base : std::max(base, self);
}

cudaError_t p3d_vort(int reg, const P3DVortProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	if (reg == int(Reg::Singular))
		return cudaMemsetAsync(p.out, 0, sizeof(float) * 3 * size_t(p.n_tgt), env.stream);
	if (use_vort_self(reg, p, env.cta_src_cap) &&
		p3d_vort_self_ws_bytes(reg, p.n_tgt, env.num_sms, env.cap_to_ws ? env.ws_bytes : 0) <=
			env.ws_bytes)
		return p3d_vort_self(reg, p, env);
	return with_vort_cfg(reg, p.n_tgt, [&](auto tag) {
		using T = decltype(tag);
		return launch_vort<T::R, T::TPT, 128, T::PK>(p, env);
	});
}

}  // namespace cvtx
