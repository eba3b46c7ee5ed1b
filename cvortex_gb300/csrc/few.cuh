// few.cuh -- the few-target form of the all-pairs kernels (the reference's
// small-target / M2S case, src/nbody.cl:258-292 and :649-684 with host-side
// partial sums), shared by the P3D, P2D and F3D launchers.
//
// CTA (x, y) takes targets [TT y, TT y + TT) and the source chunk
// [chunk_len x, chunk_len (x + 1)). Its threads stride over the chunk
// (coalesced source records) with the TT targets in registers and FP32
// partials, so every thread does useful work whatever the target count. The
// CTA then reduces every partial in FP64, by warp shuffles and then across
// warps in a fixed order, into one partial per chunk, stored target-major
// (partial[(t NC + c) n_chunks + chunk]). few_targets_finalize reduces each
// target's chunks with a whole CTA in a fixed tree and writes the result.
// Results are deterministic.
//
// An operation Op provides (all static, device side unless noted):
//   Problem, Consts           launch arguments (host types)
//   NC, NR                    output sums per target, FP32 partials per target
//   Tgt, Src                  register copies of one target / one source
//   n_src(p), n_tgt(p)
//   target(p, t), source(p, s)
//   pair(k, tgt, src, acc)    one pair into acc[NR]
//   combine(tgt, acc)         per-thread step before the reduction
//   slot(c)                   the partial that holds output sum c
//   write(p, k, t, sums)      the final outputs of target t from sums[NC]
#pragma once
#include <algorithm>
#include <cuda_runtime.h>

#include "nbody.h"
#include "plan.cuh"

namespace cvtx {

constexpr int kFewThreads = 256;
constexpr int kFewMinChunk = 8 * kFewThreads;    // sources per CTA, at least

// CVTX_GB300_FEW_MAX: the largest target count for which the few-target
// form is the built-in choice, for every operation; -1 when unset (p3d.cu).
int few_max_override();
// The P2D and F3D velocity threshold without the override: the few-target
// form beat the split form at every count up to 2,048 targets at 100,000 and
// 1,000,000 sources on GB300.
inline int few_max_targets_vel2(int) {
	const int f = few_max_override();
	return f >= 0 ? f : 2048;
}

template <class Op, int TT>
__global__ void __launch_bounds__(kFewThreads)
few_targets_kernel(const typename Op::Problem p, const typename Op::Consts k,
	double* __restrict__ partial, int chunk_len)
{
	constexpr int NC = Op::NC, NR = Op::NR;
	constexpr int kWarps = kFewThreads / 32;
	__shared__ double red[kWarps][TT * NC];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int n_tgt = Op::n_tgt(p);
	const int n_groups = (n_tgt + TT - 1) / TT;
	// target groups blockIdx.y, + gridDim.y, ... (grid.y is at most 65,535)
	for (int grp = blockIdx.y; grp < n_groups; grp += gridDim.y) {
		const int t0 = grp * TT;
		typename Op::Tgt tg[TT];
#pragma unroll
		for (int q = 0; q < TT; ++q) tg[q] = Op::target(p, t0 + q < n_tgt ? t0 + q : n_tgt - 1);
		float acc[TT][NR];
#pragma unroll
		for (int q = 0; q < TT; ++q)
#pragma unroll
			for (int c = 0; c < NR; ++c) acc[q][c] = 0.f;
		const long long s0 = (long long)blockIdx.x * chunk_len;
		long long s1 = s0 + chunk_len;
		s1 = s1 < Op::n_src(p) ? s1 : Op::n_src(p);
		for (long long s = s0 + tid; s < s1; s += kFewThreads) {
			const typename Op::Src sr = Op::source(p, s);
#pragma unroll
			for (int q = 0; q < TT; ++q) Op::pair(k, tg[q], sr, acc[q]);
		}
#pragma unroll
		for (int q = 0; q < TT; ++q) {
			Op::combine(tg[q], acc[q]);
#pragma unroll
			for (int c = 0; c < NC; ++c) {
				double v = double(acc[q][Op::slot(c)]);
#pragma unroll
				for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
				if (lane == 0) red[warp][q * NC + c] = v;
			}
		}
		__syncthreads();
		for (int i = tid; i < TT * NC; i += kFewThreads) {
			const int q = i / NC, c = i - q * NC;
			if (t0 + q >= n_tgt) continue;
			double v = 0.0;
#pragma unroll
			for (int w = 0; w < kWarps; ++w) v += red[w][i];
			partial[(size_t(t0 + q) * NC + c) * gridDim.x + blockIdx.x] = v;
		}
		__syncthreads();   // red is reused by the next group
	}
}

template <class Op>
__global__ void __launch_bounds__(kFewThreads)
few_targets_finalize(const typename Op::Problem p, const typename Op::Consts k,
	const double* __restrict__ partial, int n_chunks)
{
	constexpr int NC = Op::NC;
	constexpr int kWarps = kFewThreads / 32;
	__shared__ double red[kWarps][NC];
	const int t = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	double s[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) s[c] = 0.0;
	for (int i = tid; i < n_chunks; i += kFewThreads)
#pragma unroll
		for (int c = 0; c < NC; ++c) s[c] += partial[(size_t(t) * NC + c) * n_chunks + i];
#pragma unroll
	for (int c = 0; c < NC; ++c) {
		double v = s[c];
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
		if (lane == 0) red[warp][c] = v;
	}
	__syncthreads();
	if (tid != 0) return;
	double tot[NC];
#pragma unroll
	for (int c = 0; c < NC; ++c) {
		tot[c] = 0.0;
#pragma unroll
		for (int w = 0; w < kWarps; ++w) tot[c] += red[w][c];
	}
	Op::write(p, k, t, tot);
}

// Plan (host): n_tblocks = target groups of tt, n_split = source chunks (at
// least kFewMinChunk sources each, about two waves of CTAs of `occ` per SM,
// at most max_chunks or 4,096 when max_chunks < 0), src_per_split = chunk
// length.
inline Plan few_plan(int n_src, int n_tgt, int tt, int nc, int num_sms, int occ, int max_chunks)
{
	Plan pl;
	pl.n_tblocks = std::max(1, (n_tgt + tt - 1) / tt);
	const long long want = 2LL * num_sms * std::max(1, occ);
	long long chunks = (want + pl.n_tblocks - 1) / pl.n_tblocks;
	chunks = std::min<long long>(chunks, std::max(1, n_src / kFewMinChunk));
	chunks = std::min<long long>(chunks, max_chunks < 0 ? 4096 : max_chunks);
	chunks = std::max<long long>(chunks, 1);
	int len = int((n_src + chunks - 1) / chunks);
	len = std::max(32, (len + 31) / 32 * 32);
	pl.src_per_split = len;
	pl.n_split = std::max(1, (n_src + len - 1) / len);
	pl.smem = 0;
	pl.ws_bytes = size_t(pl.n_split) * nc * size_t(n_tgt) * sizeof(double);
	return pl;
}

// The few-target form of one operation: TT targets per CTA (one when the
// call has a single target).
template <class Op, int TT>
struct FewForm {
	static int tt(int n_tgt) { return n_tgt == 1 ? 1 : TT; }
	static int occupancy() {
		static const int occ = resident_ctas(few_targets_kernel<Op, TT>, kFewThreads, 0);
		return occ;
	}
	static Plan plan(int n_src, int n_tgt, int num_sms, int max_chunks) {
		return few_plan(n_src, n_tgt, tt(n_tgt), Op::NC, num_sms, occupancy(), max_chunks);
	}
	static cudaError_t launch(const Plan& pl, const typename Op::Problem& p,
		const typename Op::Consts& k, int n_tgt, const LaunchEnv& env) {
		if (pl.ws_bytes > env.ws_bytes) return cudaErrorInvalidValue;
		double* partial = static_cast<double*>(env.ws);
		const dim3 grid(pl.n_split, std::min(pl.n_tblocks, 65535));
		if (tt(n_tgt) == 1)
			few_targets_kernel<Op, 1><<<grid, kFewThreads, 0, env.stream>>>(p, k, partial,
				pl.src_per_split);
		else
			few_targets_kernel<Op, TT><<<grid, kFewThreads, 0, env.stream>>>(p, k, partial,
				pl.src_per_split);
		count_launch();
		few_targets_finalize<Op><<<n_tgt, kFewThreads, 0, env.stream>>>(p, k, partial, pl.n_split);
		count_launch();
		return cudaGetLastError();
	}
};

// Two group widths of one operation's few-target form: the narrow one (TTN
// targets per CTA) below 262,144 sources or up to 64 targets, else the wide
// one (TTW). Fewer targets per CTA means fewer registers and more resident
// CTAs, which hide the source loads better, until the extra target groups
// multiply the source reads (GB300 timings).
template <class Op, int TTN, int TTW>
struct FewForm2 {
	using Narrow = FewForm<Op, TTN>;
	using Wide = FewForm<Op, TTW>;
	static bool narrow(int n_src, int n_tgt) { return n_src < 262144 || n_tgt <= 64; }
	static Plan plan(int n_src, int n_tgt, int num_sms, int max_chunks) {
		return narrow(n_src, n_tgt) ? Narrow::plan(n_src, n_tgt, num_sms, max_chunks)
		                            : Wide::plan(n_src, n_tgt, num_sms, max_chunks);
	}
	static cudaError_t launch(const Plan& pl, const typename Op::Problem& p,
		const typename Op::Consts& k, int n_src, int n_tgt, const LaunchEnv& env) {
		return narrow(n_src, n_tgt) ? Narrow::launch(pl, p, k, n_tgt, env)
		                            : Wide::launch(pl, p, k, n_tgt, env);
	}
};

}  // namespace cvtx
