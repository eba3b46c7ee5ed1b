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
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include "nbody.h"
#include "plan.cuh"
#include "regfuncs.cuh"
#include "tile_stream.cuh"

namespace cvtx {

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

constexpr int kTile = 256;
constexpr int kStages = 2;
using Stream2 = TileStream<2, kTile, kStages>;

template <Reg R> struct FiniteAtZero { static constexpr bool value = true; };
template <> struct FiniteAtZero<Reg::Singular> { static constexpr bool value = false; };

struct InduceConsts {
	RegConsts rc;
	double s_vel, s_dv, k_scale;
};

RegConsts make_reg_consts(float sigma) { return make_reg_consts_host(sigma); }

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
	default:  // Winckelmans, Gaussian: rho-normalised G and K
		k.s_vel = -inv4pi / (as * as * as);
		k.s_dv = inv4pi / (s * s * s);
		k.k_scale = 1.0 / (s * s);
		break;
	}
	return k;
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
// when the cross products are.
// Shared state per target (compensated across tiles): u (3, VEL), A' and B
// (6, DV).
template <Reg R, bool VEL, bool DV, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_induce_kernel(const P3DInduceProblem p, const InduceConsts kc,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	constexpr int NC = (VEL ? 3 : 0) + (DV ? 6 : 0);     // compensated sums
	constexpr int NR = (VEL ? (DV ? 6 : 3) : 0) + (DV ? 6 : 0);  // register partials
	constexpr bool kFinite = FiniteAtZero<R>::value;
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
		float acc[NR][TPT];
#pragma unroll
		for (int c = 0; c < NR; ++c)
#pragma unroll
			for (int k = 0; k < TPT; ++k) acc[c][k] = 0.f;

		auto body = [&](int j) {
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const float dx = tx[k] - sp.x;
				const float dy = ty[k] - sp.y;
				const float dz = tz[k] - sp.z;
				const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
				if (DV) {
					const float ex = sv.x - ax[k];
					const float ey = sv.y - ay[k];
					const float ez = sv.z - az[k];
					// c' = d x da
					const float cx = fmaf(dy, ez, -dz * ey);
					const float cy = fmaf(dz, ex, -dx * ez);
					const float cz = fmaf(dx, ey, -dy * ex);
					float G, K;
					RegP3D<R>::gk(r2, kc.rc, G, K);
					const bool nz = r2 > 0.f;
					G = nz ? G : 0.f;
					if (!kFinite) K = nz ? K : 0.f;
					constexpr int o = VEL ? 6 : 0;
					if (VEL) {
						acc[0][k] = fmaf(G, cx, acc[0][k]);
						acc[1][k] = fmaf(G, cy, acc[1][k]);
						acc[2][k] = fmaf(G, cz, acc[2][k]);
						acc[3][k] = fmaf(G, dx, acc[3][k]);
						acc[4][k] = fmaf(G, dy, acc[4][k]);
						acc[5][k] = fmaf(G, dz, acc[5][k]);
					}
					acc[o + 0][k] = fmaf(G, ex, acc[o + 0][k]);
					acc[o + 1][k] = fmaf(G, ey, acc[o + 1][k]);
					acc[o + 2][k] = fmaf(G, ez, acc[o + 2][k]);
					const float pd = fmaf(az[k], cz, fmaf(ay[k], cy, ax[k] * cx));
					const float kk = K * pd;
					acc[o + 3][k] = fmaf(kk, dx, acc[o + 3][k]);
					acc[o + 4][k] = fmaf(kk, dy, acc[o + 4][k]);
					acc[o + 5][k] = fmaf(kk, dz, acc[o + 5][k]);
				} else {
					// c = d x alpha_s
					const float cx = fmaf(dy, sv.z, -dz * sv.y);
					const float cy = fmaf(dz, sv.x, -dx * sv.z);
					const float cz = fmaf(dx, sv.y, -dy * sv.x);
					float G = RegP3D<R>::g(r2, kc.rc);
					if (!kFinite) G = r2 > 0.f ? G : 0.f;
					acc[0][k] = fmaf(G, cx, acc[0][k]);
					acc[1][k] = fmaf(G, cy, acc[1][k]);
					acc[2][k] = fmaf(G, cz, acc[2][k]);
				}
			}
		};
		if (cnt == kTile) {
#pragma unroll 2
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
		if (VEL && DV) {
			// tile velocity u' + W x alpha_t into slots 0..2
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const float wx = acc[3][k], wy = acc[4][k], wz = acc[5][k];
				acc[0][k] += fmaf(wy, az[k], -wz * ay[k]);
				acc[1][k] += fmaf(wz, ax[k], -wx * az[k]);
				acc[2][k] += fmaf(wx, ay[k], -wy * ax[k]);
			}
		}
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int src_c = (VEL && DV && c >= 3) ? c + 3 : c;
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const int i = (c * TPT + k) * NT + tid;
				float h = hi[i], l = lo[i];
				fold_twosum(h, l, acc[src_c][k]);
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
			write_induce<VEL, DV>(p, kc, t, s, ax[k], ay[k], az[k]);
		} else {
#pragma unroll
			for (int c = 0; c < NC; ++c)
				partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s[c];
		}
	}
}

// Packed variant of p3d_induce_kernel for VEL+DV and DV with an even number
// of targets per thread: targets (2h, 2h+1) of a thread share one float2 lane
// pair, so every per-pair FP32 operation (except rsqrt and the coincidence
// select) is one f32x2 instruction for two interactions. Same sums, same
// order of operations per target as the scalar kernel.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

template <Reg R, bool VEL, bool DV, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_induce2_kernel(const P3DInduceProblem p, const InduceConsts kc,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	static_assert(DV && TPT % 2 == 0, "packed kernel: stretching, even TPT");
	constexpr int H = TPT / 2;
	constexpr int NC = (VEL ? 3 : 0) + 6;
	constexpr int NR = (VEL ? 6 : 0) + 6;
	constexpr bool kFinite = FiniteAtZero<R>::value;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream2::kSmemBytes);
	float* lo = hi + NC * TPT * NT;

	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
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
		float2 acc[NR][H];
#pragma unroll
		for (int c = 0; c < NR; ++c)
#pragma unroll
			for (int h = 0; h < H; ++h) acc[c][h] = make_float2(0.f, 0.f);

		auto body = [&](int j) {
			const float4 sp = st[2 * j];
			const float4 sv = st[2 * j + 1];
			const float2 nsx = bc2(-sp.x), nsy = bc2(-sp.y), nsz = bc2(-sp.z);
			const float2 wx = bc2(sv.x), wy = bc2(sv.y), wz = bc2(sv.z);
#pragma unroll
			for (int h = 0; h < H; ++h) {
				const float2 dx = __fadd2_rn(tx[h], nsx);
				const float2 dy = __fadd2_rn(ty[h], nsy);
				const float2 dz = __fadd2_rn(tz[h], nsz);
				const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
				// da = alpha_s - alpha_t, c' = d x da
				const float2 ex = __ffma2_rn(ax[h], bc2(-1.f), wx);
				const float2 ey = __ffma2_rn(ay[h], bc2(-1.f), wy);
				const float2 ez = __ffma2_rn(az[h], bc2(-1.f), wz);
				const float2 cx = __ffma2_rn(dy, ez, neg2(__fmul2_rn(dz, ey)));
				const float2 cy = __ffma2_rn(dz, ex, neg2(__fmul2_rn(dx, ez)));
				const float2 cz = __ffma2_rn(dx, ey, neg2(__fmul2_rn(dy, ex)));
				float2 G, K;
				RegP3D2<R>::gk2(r2, kc.rc, G, K);
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
		if (cnt == kTile) {
#pragma unroll 2
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
		if (VEL) {
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
			const int src_c = (VEL && c >= 3) ? c + 3 : c;
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

	if (!Stream2::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;

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
			if (gridDim.y == 1) {
				write_induce<VEL, DV>(p, kc, t, sacc, tax, tay, taz);
			} else {
#pragma unroll
				for (int c = 0; c < NC; ++c)
					partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = sacc[c];
			}
		}
	}
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
	float ax = 0.f, ay = 0.f, az = 0.f;
	if (DV) {
		const float4 tv = p.tgt[size_t(t) * p.tstride + 1];
		ax = tv.x; ay = tv.y; az = tv.z;
	}
	write_induce<VEL, DV>(p, kc, t, s, ax, ay, az);
}

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
template <Reg R> struct ZetaP3D;
template <> struct ZetaP3D<Reg::Singular> {
	__device__ __forceinline__ static float z(float, const RegConsts&) { return 0.f; } };
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
				const bool in = fabsf(dx) < cutoff && fabsf(dy) < cutoff && fabsf(dz) < cutoff;
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

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <int TPT, int NT, int NC>
constexpr size_t smem_bytes() {
	return Stream2::kSmemBytes + size_t(2) * NC * TPT * NT * sizeof(float);
}

// Targets per CTA: large problems use 4 targets per thread; small target
// counts use 1 so that the source dimension can be split across more CTAs.
constexpr int kSmallTargets = 8192;

// Packed (f32x2) kernel for stretching with an even number of targets per
// thread; CVTX_GB300_SCALAR=1 in the environment selects the scalar kernel
// (kept for comparison).
bool use_packed() {
	static const bool v = [] {
		const char* e = std::getenv("CVTX_GB300_SCALAR");
		return !(e && e[0] == '1');
	}();
	return v;
}

template <Reg R, bool VEL, bool DV, int TPT, int NT>
struct InduceKernel {
	using Fn = void (*)(const P3DInduceProblem, const InduceConsts, double*, int, unsigned*);
	static constexpr bool kPackable = DV && (TPT % 2 == 0);
	static Fn get() {
		if constexpr (kPackable) {
			if (use_packed()) return p3d_induce2_kernel<R, VEL, DV, TPT, NT>;
		}
		return p3d_induce_kernel<R, VEL, DV, TPT, NT>;
	}
};

template <Reg R, bool VEL, bool DV, int TPT, int NT>
Plan plan_induce(int n_src, int n_tgt, int num_sms) {
	constexpr int NC = (VEL ? 3 : 0) + (DV ? 6 : 0);
	constexpr size_t smem = smem_bytes<TPT, NT, NC>();
	static const int occ = resident_ctas(InduceKernel<R, VEL, DV, TPT, NT>::get(), NT, smem);
	return make_plan(n_src, n_tgt, TPT * NT, kTile, NC, num_sms * occ, smem);
}

template <Reg R, bool VEL, bool DV, int TPT, int NT>
cudaError_t launch_induce(const P3DInduceProblem& p, const LaunchEnv& env) {
	constexpr int NC = (VEL ? 3 : 0) + (DV ? 6 : 0);
	const Plan pl = plan_induce<R, VEL, DV, TPT, NT>(p.n_src, p.n_tgt, env.num_sms);
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	const InduceConsts kc = make_induce_consts(int(R), p.sigma);
	double* partial = static_cast<double*>(env.ws);
	dim3 grid(pl.n_tblocks, pl.n_split);
	InduceKernel<R, VEL, DV, TPT, NT>::get()<<<grid, NT, pl.smem, env.stream>>>(
		p, kc, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		p3d_induce_finalize<VEL, DV><<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
			p, kc, partial, pl.n_split);
		count_launch();
	}
	(void)NC;
	return cudaGetLastError();
}

template <Reg R, bool VEL, bool DV>
size_t ws_induce_r(int n_src, int n_tgt, int num_sms) {
	if (n_tgt < kSmallTargets) return plan_induce<R, VEL, DV, 1, 128>(n_src, n_tgt, num_sms).ws_bytes;
	return plan_induce<R, VEL, DV, 4, 128>(n_src, n_tgt, num_sms).ws_bytes;
}

template <Reg R, bool VEL, bool DV>
cudaError_t induce_r(const P3DInduceProblem& p, const LaunchEnv& env) {
	if (p.n_tgt < kSmallTargets) return launch_induce<R, VEL, DV, 1, 128>(p, env);
	return launch_induce<R, VEL, DV, 4, 128>(p, env);
}

template <Reg R>
size_t ws_induce_ops(unsigned ops, int n_src, int n_tgt, int num_sms) {
	switch (ops) {
	case kOpVel: return ws_induce_r<R, true, false>(n_src, n_tgt, num_sms);
	case kOpDvort: return ws_induce_r<R, false, true>(n_src, n_tgt, num_sms);
	default: return ws_induce_r<R, true, true>(n_src, n_tgt, num_sms);
	}
}

template <Reg R>
cudaError_t induce_ops(unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env) {
	switch (ops) {
	case kOpVel: return induce_r<R, true, false>(p, env);
	case kOpDvort: return induce_r<R, false, true>(p, env);
	default: return induce_r<R, true, true>(p, env);
	}
}

// The same launch with the number of source splits capped so that the FP64
// split partials fit the workspace the caller supplies (env.ws_bytes), for
// callers that provide a fixed scratch area instead of a sized one.
template <Reg R, bool VEL, bool DV, int TPT, int NT>
cudaError_t launch_induce_bounded(const P3DInduceProblem& p, const LaunchEnv& env) {
	constexpr int NC = (VEL ? 3 : 0) + (DV ? 6 : 0);
	constexpr size_t smem = smem_bytes<TPT, NT, NC>();
	static const int occ = resident_ctas(InduceKernel<R, VEL, DV, TPT, NT>::get(), NT, smem);
	const size_t per_split = size_t(NC) * size_t(p.n_tgt) * sizeof(double);
	size_t cap = env.ws_bytes / per_split;
	cap = cap < 1 ? 1 : (cap > 64 ? 64 : cap);
	const Plan pl = make_plan(p.n_src, p.n_tgt, TPT * NT, kTile, NC, env.num_sms * occ, smem,
		int(cap));
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	const InduceConsts kc = make_induce_consts(int(R), p.sigma);
	double* partial = static_cast<double*>(env.ws);
	InduceKernel<R, VEL, DV, TPT, NT>::get()<<<dim3(pl.n_tblocks, pl.n_split), NT, pl.smem,
		env.stream>>>(p, kc, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		p3d_induce_finalize<VEL, DV><<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
			p, kc, partial, pl.n_split);
		count_launch();
	}
	return cudaGetLastError();
}

template <Reg R, bool VEL, bool DV>
cudaError_t induce_bounded_r(const P3DInduceProblem& p, const LaunchEnv& env) {
	if (p.n_tgt < kSmallTargets) return launch_induce_bounded<R, VEL, DV, 1, 128>(p, env);
	return launch_induce_bounded<R, VEL, DV, 4, 128>(p, env);
}

template <Reg R>
cudaError_t induce_bounded_ops(unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env) {
	switch (ops) {
	case kOpVel: return induce_bounded_r<R, true, false>(p, env);
	case kOpDvort: return induce_bounded_r<R, false, true>(p, env);
	default: return induce_bounded_r<R, true, true>(p, env);
	}
}

template <Reg R, int TPT, int NT>
Plan plan_visc(int n_src, int n_tgt, int num_sms) {
	constexpr size_t smem = smem_bytes<TPT, NT, 3>();
	static const int occ = resident_ctas(p3d_visc_kernel<R, TPT, NT>, NT, smem);
	return make_plan(n_src, n_tgt, TPT * NT, kTile, 3, num_sms * occ, smem);
}

template <Reg R, int TPT, int NT>
cudaError_t launch_visc(const P3DViscProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_visc<R, TPT, NT>(p.n_src, p.n_tgt, env.num_sms);
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	ViscConsts vc;
	vc.rc = make_reg_consts(p.sigma);
	const double base = 2.0 * double(p.nu) / (double(p.sigma) * double(p.sigma));
	vc.scale = base * (R == Reg::Winckelmans ? 52.5 : double(kSqrt2OverPi));
	double* partial = static_cast<double*>(env.ws);
	dim3 grid(pl.n_tblocks, pl.n_split);
	p3d_visc_kernel<R, TPT, NT><<<grid, NT, pl.smem, env.stream>>>(
		p, vc, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		p3_finalize_scaled<<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
			p.out, p.n_tgt, partial, pl.n_split, vc.scale);
		count_launch();
	}
	return cudaGetLastError();
}

template <Reg R, int TPT, int NT>
Plan plan_vort(int n_src, int n_tgt, int num_sms) {
	constexpr size_t smem = smem_bytes<TPT, NT, 3>();
	static const int occ = resident_ctas(p3d_vort_kernel<R, TPT, NT>, NT, smem);
	return make_plan(n_src, n_tgt, TPT * NT, kTile, 3, num_sms * occ, smem);
}

template <Reg R, int TPT, int NT>
cudaError_t launch_vort(const P3DVortProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_vort<R, TPT, NT>(p.n_src, p.n_tgt, env.num_sms);
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	const RegConsts rc = make_reg_consts(p.sigma);
	const double s = p.sigma;
	const double scale = 1.0 / (4.0 * 3.14159265358979323846 * s * s * s);
	const float cutoff = 5.f * p.sigma;
	double* partial = static_cast<double*>(env.ws);
	dim3 grid(pl.n_tblocks, pl.n_split);
	p3d_vort_kernel<R, TPT, NT><<<grid, NT, pl.smem, env.stream>>>(
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

size_t p3d_induce_ws_bytes(int reg, unsigned ops, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	switch (reg) {
	case 0: return ws_induce_ops<Reg::Singular>(ops, n_src, n_tgt, num_sms);
	case 1: return ws_induce_ops<Reg::Winckelmans>(ops, n_src, n_tgt, num_sms);
	case 2: return ws_induce_ops<Reg::Planetary>(ops, n_src, n_tgt, num_sms);
	default: return ws_induce_ops<Reg::Gaussian>(ops, n_src, n_tgt, num_sms);
	}
}

cudaError_t p3d_induce(int reg, unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	switch (reg) {
	case 0: return induce_ops<Reg::Singular>(ops, p, env);
	case 1: return induce_ops<Reg::Winckelmans>(ops, p, env);
	case 2: return induce_ops<Reg::Planetary>(ops, p, env);
	case 3: return induce_ops<Reg::Gaussian>(ops, p, env);
	default: return cudaErrorInvalidValue;
	}
}

cudaError_t p3d_induce_bounded(int reg, unsigned ops, const P3DInduceProblem& p,
	const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	switch (reg) {
	case 0: return induce_bounded_ops<Reg::Singular>(ops, p, env);
	case 1: return induce_bounded_ops<Reg::Winckelmans>(ops, p, env);
	case 2: return induce_bounded_ops<Reg::Planetary>(ops, p, env);
	case 3: return induce_bounded_ops<Reg::Gaussian>(ops, p, env);
	default: return cudaErrorInvalidValue;
	}
}

size_t p3d_visc_ws_bytes(int reg, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	const bool small = n_tgt < kSmallTargets;
	if (reg == int(Reg::Winckelmans))
		return small ? plan_visc<Reg::Winckelmans, 1, 128>(n_src, n_tgt, num_sms).ws_bytes
		             : plan_visc<Reg::Winckelmans, 4, 128>(n_src, n_tgt, num_sms).ws_bytes;
	if (reg == int(Reg::Gaussian))
		return small ? plan_visc<Reg::Gaussian, 1, 128>(n_src, n_tgt, num_sms).ws_bytes
		             : plan_visc<Reg::Gaussian, 4, 128>(n_src, n_tgt, num_sms).ws_bytes;
	return 0;
}

// Only Winckelmans and Gaussian have an eta function; the runtime handles the
// other regularisations (zeros and a warning) without launching anything.
cudaError_t p3d_visc(int reg, const P3DViscProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	const bool small = p.n_tgt < kSmallTargets;
	if (reg == int(Reg::Winckelmans))
		return small ? launch_visc<Reg::Winckelmans, 1, 128>(p, env)
		             : launch_visc<Reg::Winckelmans, 4, 128>(p, env);
	if (reg == int(Reg::Gaussian))
		return small ? launch_visc<Reg::Gaussian, 1, 128>(p, env)
		             : launch_visc<Reg::Gaussian, 4, 128>(p, env);
	return cudaErrorInvalidValue;
}

size_t p3d_vort_ws_bytes(int reg, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	switch (reg) {
	case 0: return plan_vort<Reg::Singular, 4, 128>(n_src, n_tgt, num_sms).ws_bytes;
	case 1: return plan_vort<Reg::Winckelmans, 4, 128>(n_src, n_tgt, num_sms).ws_bytes;
	case 2: return plan_vort<Reg::Planetary, 4, 128>(n_src, n_tgt, num_sms).ws_bytes;
	default: return plan_vort<Reg::Gaussian, 4, 128>(n_src, n_tgt, num_sms).ws_bytes;
	}
}

cudaError_t p3d_vort(int reg, const P3DVortProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	switch (reg) {
	case 0: return launch_vort<Reg::Singular, 4, 128>(p, env);
	case 1: return launch_vort<Reg::Winckelmans, 4, 128>(p, env);
	case 2: return launch_vort<Reg::Planetary, 4, 128>(p, env);
	case 3: return launch_vort<Reg::Gaussian, 4, 128>(p, env);
	default: return cudaErrorInvalidValue;
	}
}

}  // namespace cvtx
