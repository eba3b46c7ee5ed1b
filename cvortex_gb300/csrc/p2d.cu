// p2d.cu -- all-pairs 2D vortex particle kernels for sm_103a.
//
// Replaces cvtx_nb_P2D_{vel,smallmes_vel,visc_dvort}_* (reference
// src/nbody.cl:220-338, 547-605) and src/ocl_P2D.cpp. Results follow the
// reference CPU path src/P2D.cpp:49-69 (velocity) and :167-194 (viscous
// exchange). Same CTA shape as p3d.cu; a P2D source record is one float4
// (x, y, Gamma, area), so a 512-record tile is 8 KB.
#include <cstdint>
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include "nbody.h"
#include "plan.cuh"
#include "regfuncs.cuh"
#include "tile_stream.cuh"
#include "few.cuh"

namespace cvtx {
RegConsts make_reg_consts_host(float sigma);

namespace {

constexpr int kTile = 512;
constexpr int kStages = 2;
using Stream1 = TileStream<1, kTile, kStages>;
constexpr int kSmallTargets = 8192;

template <Reg R> struct HFinite { static constexpr bool value = true; };
template <> struct HFinite<Reg::Singular> { static constexpr bool value = false; };

// Velocity: out = S * sum_s Hs Gamma_s (dy, -dx), d = x_t - x_s.
template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p2d_vel_kernel(const P2DVelProblem p, const RegConsts rc, double scale,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	constexpr int NC = 2;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream1::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float tx[TPT], ty[TPT];
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		int t = tbase + k * NT + tid;
		t = t < p.n_tgt ? t : p.n_tgt - 1;
		const float4 tp = p.tgt[t];
		tx[k] = tp.x; ty[k] = tp.y;
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
			const float4 s = st[j];
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const float dx = tx[k] - s.x;
				const float dy = ty[k] - s.y;
				const float r2 = fmaf(dy, dy, dx * dx);
				float h = RegP2D<R>::h(r2, rc);
				if (!HFinite<R>::value) h = r2 > 0.f ? h : 0.f;
				const float hg = h * s.z;
				acc[0][k] = fmaf(hg, dy, acc[0][k]);
				acc[1][k] = fmaf(-hg, dx, acc[1][k]);
			}
		};
		if (cnt == kTile) {
#pragma unroll 4
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
	if (!Stream1::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double s = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[2 * size_t(t) + c] = float(scale * s);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = s;
		}
	}
}

// Packed velocity kernel: targets 2h and 2h+1 of a thread share one f32x2
// lane pair (as the P3D packed kernel), 1/x from rcp + one Newton step.
template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p2d_vel2_kernel(const P2DVelProblem p, const RegConsts rc, double scale,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int NC = 2, H = TPT / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream1::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float2 tx[H], ty[H];
#pragma unroll
	for (int h = 0; h < H; ++h) {
		float4 q[2];
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			int t = tbase + (2 * h + e) * NT + tid;
			t = t < p.n_tgt ? t : p.n_tgt - 1;
			q[e] = p.tgt[t];
		}
		tx[h] = make_float2(q[0].x, q[1].x);
		ty[h] = make_float2(q[0].y, q[1].y);
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
			const float4 s = st[j];
			const float2 nsx = bc2(-s.x), nsy = bc2(-s.y), g = bc2(s.z);
#pragma unroll
			for (int h = 0; h < H; ++h) {
				const float2 dx = __fadd2_rn(tx[h], nsx);
				const float2 dy = __fadd2_rn(ty[h], nsy);
				const float2 r2 = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
				float2 hh = RegP2D2<R>::h2(r2, rc);
				if (!HFinite<R>::value) {
					hh.x = r2.x > 0.f ? hh.x : 0.f;
					hh.y = r2.y > 0.f ? hh.y : 0.f;
				}
				const float2 hg = __fmul2_rn(hh, g);
				acc[0][h] = __ffma2_rn(hg, dy, acc[0][h]);
				acc[1][h] = __ffma2_rn(make_float2(-hg.x, -hg.y), dx, acc[1][h]);
			}
		};
		if (cnt == kTile) {
#pragma unroll 4
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
	if (!Stream1::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
#pragma unroll
		for (int c = 0; c < NC; ++c) {
			const int i = (c * TPT + k) * NT + tid;
			const double sum = double(hi[i]) + double(lo[i]);
			if (gridDim.y == 1) p.out[2 * size_t(t) + c] = float(scale * sum);
			else partial[(size_t(blockIdx.y) * NC + c) * p.n_tgt + t] = sum;
		}
	}
}

// Viscous exchange: out = S * sum_s Es (Gamma_s A_t - Gamma_t A_s).
template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p2d_visc_kernel(const P2DViscProblem p, const RegConsts rc, double scale,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	constexpr int NC = 1;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream1::kSmemBytes);
	float* lo = hi + NC * TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float tx[TPT], ty[TPT], tg[TPT], ta[TPT];
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		int t = tbase + k * NT + tid;
		t = t < p.n_tgt ? t : p.n_tgt - 1;
		const float4 tp = p.tgt[t];
		tx[k] = tp.x; ty[k] = tp.y; tg[k] = tp.z; ta[k] = tp.w;
	}
#pragma unroll
	for (int i = 0; i < NC * TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }
	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float acc[TPT];
#pragma unroll
		for (int k = 0; k < TPT; ++k) acc[k] = 0.f;
		auto body = [&](int j) {
			const float4 s = st[j];
#pragma unroll
			for (int k = 0; k < TPT; ++k) {
				const float dx = s.x - tx[k];
				const float dy = s.y - ty[k];
				const float r2 = fmaf(dy, dy, dx * dx);
				float e = RegP2D<R>::eta(r2, rc);
				e = r2 > 0.f ? e : 0.f;
				const float w = fmaf(s.z, ta[k], -tg[k] * s.w);
				acc[k] = fmaf(e, w, acc[k]);
			}
		};
		if (cnt == kTile) {
#pragma unroll 4
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int k = 0; k < TPT; ++k) {
			const int i = k * NT + tid;
			float h = hi[i], l = lo[i];
			fold_twosum(h, l, acc[k]);
			hi[i] = h; lo[i] = l;
		}
	};
	if (!Stream1::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
		const int i = k * NT + tid;
		const double s = double(hi[i]) + double(lo[i]);
		if (gridDim.y == 1) p.out[t] = float(scale * s);
		else partial[size_t(blockIdx.y) * p.n_tgt + t] = s;
	}
}

// Packed viscous exchange (two targets per f32x2 lane pair).
template <Reg R, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p2d_visc2_kernel(const P2DViscProblem p, const RegConsts rc, double scale,
	double* __restrict__ partial, int src_per_split, unsigned* err)
{
	static_assert(TPT % 2 == 0, "packed kernel: even TPT");
	constexpr int H = TPT / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	float* hi = reinterpret_cast<float*>(smem + Stream1::kSmemBytes);
	float* lo = hi + TPT * NT;
	const int tid = threadIdx.x;
	const int tbase = blockIdx.x * (TPT * NT);
	const int s_begin = blockIdx.y * src_per_split;
	int n_s = p.n_src - s_begin;
	n_s = n_s < src_per_split ? n_s : src_per_split;
	n_s = n_s > 0 ? n_s : 0;
	float2 ntx[H], nty[H], ntg[H], ta[H];
#pragma unroll
	for (int h = 0; h < H; ++h) {
		float4 q[2];
#pragma unroll
		for (int e = 0; e < 2; ++e) {
			int t = tbase + (2 * h + e) * NT + tid;
			t = t < p.n_tgt ? t : p.n_tgt - 1;
			q[e] = p.tgt[t];
		}
		ntx[h] = make_float2(-q[0].x, -q[1].x); nty[h] = make_float2(-q[0].y, -q[1].y);
		ntg[h] = make_float2(-q[0].z, -q[1].z); ta[h] = make_float2(q[0].w, q[1].w);
	}
#pragma unroll
	for (int i = 0; i < TPT; ++i) { hi[i * NT + tid] = 0.f; lo[i * NT + tid] = 0.f; }
	auto tile_fn = [&](const float4* __restrict__ st, int cnt) {
		float2 acc[H];
#pragma unroll
		for (int h = 0; h < H; ++h) acc[h] = make_float2(0.f, 0.f);
		auto body = [&](int j) {
			const float4 s = st[j];
			const float2 sx = bc2(s.x), sy = bc2(s.y), sg = bc2(s.z), sa = bc2(s.w);
#pragma unroll
			for (int h = 0; h < H; ++h) {
				const float2 dx = __fadd2_rn(sx, ntx[h]);
				const float2 dy = __fadd2_rn(sy, nty[h]);
				const float2 r2 = __ffma2_rn(dy, dy, __fmul2_rn(dx, dx));
				float2 e = RegEta2D2<R>::eta2(r2, rc);
				e.x = r2.x > 0.f ? e.x : 0.f;
				e.y = r2.y > 0.f ? e.y : 0.f;
				// Gamma_s A_t - Gamma_t A_s
				const float2 w = __ffma2_rn(sg, ta[h], __fmul2_rn(ntg[h], sa));
				acc[h] = __ffma2_rn(e, w, acc[h]);
			}
		};
		if (cnt == kTile) {
#pragma unroll 4
			for (int j = 0; j < kTile; ++j) body(j);
		} else {
#pragma unroll 1
			for (int j = 0; j < cnt; ++j) body(j);
		}
#pragma unroll
		for (int h = 0; h < H; ++h)
#pragma unroll
			for (int e = 0; e < 2; ++e) {
				const int i = (2 * h + e) * NT + tid;
				float hv = hi[i], lv = lo[i];
				fold_twosum(hv, lv, e == 0 ? acc[h].x : acc[h].y);
				hi[i] = hv; lo[i] = lv;
			}
	};
	if (!Stream1::run(smem, p.src, s_begin, n_s, err, tile_fn)) return;
#pragma unroll
	for (int k = 0; k < TPT; ++k) {
		const int t = tbase + k * NT + tid;
		if (t >= p.n_tgt) continue;
		const int i = k * NT + tid;
		const double sum = double(hi[i]) + double(lo[i]);
		if (gridDim.y == 1) p.out[t] = float(scale * sum);
		else partial[size_t(blockIdx.y) * p.n_tgt + t] = sum;
	}
}

template <int NC>
__global__ void finalize_scaled(float* __restrict__ out, int n_tgt,
	const double* __restrict__ partial, int n_split, double scale)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n_tgt) return;
	double s[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) s[c] = 0.0;
	for (int sp = 0; sp < n_split; ++sp)
#pragma unroll
		for (int c = 0; c < NC; ++c) s[c] += partial[(size_t(sp) * NC + c) * n_tgt + t];
#pragma unroll
	for (int c = 0; c < NC; ++c) out[NC * size_t(t) + c] = float(scale * s[c]);
}

template <int TPT, int NT, int NC>
constexpr size_t smem_bytes() {
	return Stream1::kSmemBytes + size_t(2) * NC * TPT * NT * sizeof(float);
}

template <Reg R, int TPT, int NT, bool PK>
auto vel_kernel() {
	if constexpr (PK) return p2d_vel2_kernel<R, TPT, NT>;
	else return p2d_vel_kernel<R, TPT, NT>;
}

template <Reg R, int TPT, int NT, bool PK>
Plan plan_vel(int n_src, int n_tgt, int num_sms, int max_split = 64, int min_split = 1) {
	constexpr size_t smem = smem_bytes<TPT, NT, 2>();
	static const int occ = resident_ctas(vel_kernel<R, TPT, NT, PK>(), NT, smem);
	return make_plan(n_src, n_tgt, TPT * NT, kTile, 2, num_sms * occ, smem, max_split, min_split);
}

// Reference scale 1/(2 pi) (src/P2D.cpp:118); Winckelmans and Gaussian H are
// rho-normalised and carry an extra 1/sigma^2.
double vel_scale(int reg, float sigma) {
	const double inv2pi = 1.0 / (2.0 * 3.14159265358979323846);
	if (reg == int(Reg::Winckelmans) || reg == int(Reg::Gaussian))
		return inv2pi / (double(sigma) * double(sigma));
	return inv2pi;
}

template <Reg R, int TPT, int NT, bool PK>
cudaError_t launch_vel(const P2DVelProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_vel<R, TPT, NT, PK>(p.n_src, p.n_tgt, env.num_sms,
		env.cap_to_ws ? split_cap_for(env.ws_bytes, 2, p.n_tgt) : 64, min_split_for(env, p.n_src));
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	const RegConsts rc = make_reg_consts_host(p.sigma);
	const double scale = vel_scale(int(R), p.sigma);
	double* partial = static_cast<double*>(env.ws);
	vel_kernel<R, TPT, NT, PK>()<<<dim3(pl.n_tblocks, pl.n_split), NT, pl.smem, env.stream>>>(
		p, rc, scale, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		finalize_scaled<2><<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
			p.out, p.n_tgt, partial, pl.n_split, scale);
		count_launch();
	}
	return cudaGetLastError();
}

template <Reg R, int TPT, int NT, bool PK>
auto visc_kernel() {
	if constexpr (PK) return p2d_visc2_kernel<R, TPT, NT>;
	else return p2d_visc_kernel<R, TPT, NT>;
}

template <Reg R, int TPT, int NT, bool PK>
Plan plan_visc(int n_src, int n_tgt, int num_sms, int max_split = 64) {
	constexpr size_t smem = smem_bytes<TPT, NT, 1>();
	static const int occ = resident_ctas(visc_kernel<R, TPT, NT, PK>(), NT, smem);
	return make_plan(n_src, n_tgt, TPT * NT, kTile, 1, num_sms * occ, smem, max_split);
}

template <Reg R, int TPT, int NT, bool PK>
cudaError_t launch_visc(const P2DViscProblem& p, const LaunchEnv& env) {
	const Plan pl = plan_visc<R, TPT, NT, PK>(p.n_src, p.n_tgt, env.num_sms,
		env.cap_to_ws ? split_cap_for(env.ws_bytes, 1, p.n_tgt) : 64);
	if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
	const RegConsts rc = make_reg_consts_host(p.sigma);
	const double scale = 2.0 * double(p.nu) / (double(p.sigma) * double(p.sigma));
	double* partial = static_cast<double*>(env.ws);
	visc_kernel<R, TPT, NT, PK>()<<<dim3(pl.n_tblocks, pl.n_split), NT, pl.smem, env.stream>>>(
		p, rc, scale, partial, pl.src_per_split, env.err);
	count_launch();
	if (pl.n_split > 1) {
		finalize_scaled<1><<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(
			p.out, p.n_tgt, partial, pl.n_split, scale);
		count_launch();
	}
	return cudaGetLastError();
}

// Velocity launch configurations: 0 scalar (1 target/thread, 128 threads),
// 1 scalar (4, 128), 2 packed (4, 128), 3 packed (2, 128), 4 packed (8, 128),
// 5 packed (4, 256), 6 the few-target form. Default from GB300 timings
// (Gaussian patch, 20,000 and 200,000 targets): 6 up to
// few_max_targets_vel2() targets, 0 below kSmallTargets, 3 up to 65,535,
// else 2;
// CVTX_GB300_P2D_CFG forces one.
constexpr int kP2DFewCfg = 6;   // the few-target form (few.cuh)
int p2d_env_cfg() {
	static const int v = [] {
		const char* e = std::getenv("CVTX_GB300_P2D_CFG");
		if (!e || !*e) return -1;
		const int c = std::atoi(e);
		return (c >= 0 && c <= kP2DFewCfg) ? c : -1;
	}();
	return v;
}
// The P2D velocity pair as an operation of the few-target form (few.cuh):
// the same per-pair arithmetic as p2d_vel_kernel.
template <Reg R>
struct P2DVelOp {
	using Problem = P2DVelProblem;
	struct Consts { RegConsts rc; double scale; };
	static constexpr int NC = 2, NR = 2;
	struct Tgt { float x, y; };
	using Src = float4;
	__device__ static int n_src(const Problem& p) { return p.n_src; }
	__device__ static int n_tgt(const Problem& p) { return p.n_tgt; }
	__device__ static Tgt target(const Problem& p, int t) { const float4 q = p.tgt[t]; return Tgt{q.x, q.y}; }
	__device__ static Src source(const Problem& p, long long s) { return p.src[s]; }
	__device__ static void pair(const Consts& k, const Tgt& t, const Src& s, float (&acc)[NR]) {
		const float dx = t.x - s.x;
		const float dy = t.y - s.y;
		const float r2 = fmaf(dy, dy, dx * dx);
		float h = RegP2D<R>::h(r2, k.rc);
		if (!HFinite<R>::value) h = r2 > 0.f ? h : 0.f;
		const float hg = h * s.z;
		acc[0] = fmaf(hg, dy, acc[0]);
		acc[1] = fmaf(-hg, dx, acc[1]);
	}
	__device__ static void combine(const Tgt&, float (&)[NR]) {}
	__device__ static int slot(int c) { return c; }
	__device__ static void write(const Problem& p, const Consts& k, int t, const double* s) {
		p.out[2 * size_t(t)] = float(k.scale * s[0]);
		p.out[2 * size_t(t) + 1] = float(k.scale * s[1]);
	}
};
template <Reg R> using P2DFew = FewForm2<P2DVelOp<R>, 4, 8>;

int vel_cfg(int n_tgt, int n_src) {
	const int f = p2d_env_cfg();
	if (f >= 0) return f;
	if (n_tgt <= few_max_targets_vel2(n_src)) return kP2DFewCfg;
	return n_tgt < kSmallTargets ? 0 : n_tgt < 65536 ? 3 : 2;
}
template <Reg R, class F>
auto with_vel_cfg(int cfg, F&& f) {
	switch (cfg) {
	case 0: return f(std::integral_constant<int, 1>{}, std::integral_constant<int, 128>{}, std::false_type{});
	case 1: return f(std::integral_constant<int, 4>{}, std::integral_constant<int, 128>{}, std::false_type{});
	case 2: return f(std::integral_constant<int, 4>{}, std::integral_constant<int, 128>{}, std::true_type{});
	case 3: return f(std::integral_constant<int, 2>{}, std::integral_constant<int, 128>{}, std::true_type{});
	case 4: return f(std::integral_constant<int, 8>{}, std::integral_constant<int, 128>{}, std::true_type{});
	default: return f(std::integral_constant<int, 4>{}, std::integral_constant<int, 256>{}, std::true_type{});
	}
}
template <Reg R>
size_t ws_vel_r(int n_src, int n_tgt, int num_sms) {
	if (vel_cfg(n_tgt, n_src) == kP2DFewCfg)
		return P2DFew<R>::plan(n_src, n_tgt, num_sms, -1).ws_bytes;
	return with_vel_cfg<R>(vel_cfg(n_tgt, n_src), [&](auto t, auto n, auto pk) {
		return plan_vel<R, decltype(t)::value, decltype(n)::value, decltype(pk)::value>(
			n_src, n_tgt, num_sms).ws_bytes;
	});
}
template <Reg R>
cudaError_t vel_r(const P2DVelProblem& p, const LaunchEnv& env) {
	if (vel_cfg(p.n_tgt, p.n_src) == kP2DFewCfg) {
		const Plan pl = P2DFew<R>::plan(p.n_src, p.n_tgt, env.num_sms,
			env.cap_to_ws ? split_cap_for(env.ws_bytes, 2, p.n_tgt) : -1);
		typename P2DVelOp<R>::Consts k{make_reg_consts_host(p.sigma), vel_scale(int(R), p.sigma)};
		return P2DFew<R>::launch(pl, p, k, p.n_src, p.n_tgt, env);
	}
	return with_vel_cfg<R>(vel_cfg(p.n_tgt, p.n_src), [&](auto t, auto n, auto pk) {
		return launch_vel<R, decltype(t)::value, decltype(n)::value, decltype(pk)::value>(p, env);
	});
}
template <Reg R>
size_t ws_visc_r(int n_src, int n_tgt, int num_sms) {
	return n_tgt < kSmallTargets ? plan_visc<R, 1, 128, false>(n_src, n_tgt, num_sms).ws_bytes
	                             : plan_visc<R, 4, 128, true>(n_src, n_tgt, num_sms).ws_bytes;
}
template <Reg R>
cudaError_t visc_r(const P2DViscProblem& p, const LaunchEnv& env) {
	return p.n_tgt < kSmallTargets ? launch_visc<R, 1, 128, false>(p, env)
	                               : launch_visc<R, 4, 128, true>(p, env);
}

}  // namespace

double p2d_vel_scale(int reg, float sigma) { return vel_scale(reg, sigma); }

static bool use_vel_self(const P2DVelProblem& p, int cta_src_cap) {
	return cta_src_cap == 0 && p2d_env_cfg() < 0 && p2d_vel_self_form_applies(p);
}

size_t p2d_vel_ws_bytes_for(int reg, const P2DVelProblem& p, int num_sms) {
	if (p.n_tgt <= 0) return 0;
	const size_t base = p2d_vel_ws_bytes(reg, p.n_src, p.n_tgt, num_sms);
	if (!use_vel_self(p, 0)) return base;
	const size_t self = p2d_vel_self_ws_bytes(reg, p.n_tgt, num_sms);
	return self == SIZE_MAX ? base : std::max(base, self);
}

size_t p2d_visc_ws_bytes_for(int reg, const P2DViscProblem& p, int num_sms) {
	if (p.n_tgt <= 0) return 0;
	const size_t base = p2d_visc_ws_bytes(reg, p.n_src, p.n_tgt, num_sms);
	if (!p2d_visc_self_form_applies(reg, p)) return base;
	const size_t self = p2d_visc_self_ws_bytes(reg, p.n_tgt, num_sms);
	return self == SIZE_MAX ? base : std::max(base, self);
}

size_t p2d_vel_ws_bytes(int reg, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	switch (reg) {
	case 0: return ws_vel_r<Reg::Singular>(n_src, n_tgt, num_sms);
	case 1: return ws_vel_r<Reg::Winckelmans>(n_src, n_tgt, num_sms);
	case 2: return ws_vel_r<Reg::Planetary>(n_src, n_tgt, num_sms);
	default: return ws_vel_r<Reg::Gaussian>(n_src, n_tgt, num_sms);
	}
}

cudaError_t p2d_vel(int reg, const P2DVelProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	if (reg >= 0 && reg <= 3 && use_vel_self(p, env.cta_src_cap) &&
		p2d_vel_self_ws_bytes(reg, p.n_tgt, env.num_sms, env.cap_to_ws ? env.ws_bytes : 0) <=
			env.ws_bytes)
		return p2d_vel_self(reg, p, env);
	switch (reg) {
	case 0: return vel_r<Reg::Singular>(p, env);
	case 1: return vel_r<Reg::Winckelmans>(p, env);
	case 2: return vel_r<Reg::Planetary>(p, env);
	case 3: return vel_r<Reg::Gaussian>(p, env);
	default: return cudaErrorInvalidValue;
	}
}

size_t p2d_visc_ws_bytes(int reg, int n_src, int n_tgt, int num_sms) {
	if (n_tgt <= 0) return 0;
	if (reg == int(Reg::Winckelmans)) return ws_visc_r<Reg::Winckelmans>(n_src, n_tgt, num_sms);
	if (reg == int(Reg::Gaussian)) return ws_visc_r<Reg::Gaussian>(n_src, n_tgt, num_sms);
	return 0;
}

cudaError_t p2d_visc(int reg, const P2DViscProblem& p, const LaunchEnv& env) {
	if (p.n_tgt <= 0) return cudaSuccess;
	if (env.cta_src_cap == 0 && p2d_visc_self_form_applies(reg, p) &&
		p2d_visc_self_ws_bytes(reg, p.n_tgt, env.num_sms, env.cap_to_ws ? env.ws_bytes : 0) <=
			env.ws_bytes)
		return p2d_visc_self(reg, p, env);
	if (reg == int(Reg::Winckelmans)) return visc_r<Reg::Winckelmans>(p, env);
	if (reg == int(Reg::Gaussian)) return visc_r<Reg::Gaussian>(p, env);
	return cudaErrorInvalidValue;
}

}  // namespace cvtx
