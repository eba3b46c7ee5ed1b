// sym.cuh -- pair interactions of a particle set with itself, each unordered
// pair evaluated once (the self-interaction form), for any pair operation
// whose two terms are related: the operations are in p3d_sym.cu (P3D
// velocity / stretching / viscous exchange) and p2d_sym.cu (P2D velocity /
// viscous exchange).
//
// Work decomposition (deterministic, no floating-point atomics):
// * The particles are cut into nb blocks of S (a multiple of the 512-particle
//   pass of a CTA; the last block may be shorter). A work item is a block
//   pair (bi, bj), bi <= bj; a persistent grid claims items through an atomic
//   counter, largest first.
// * Item (bi, bj), bi < bj: for each pass of 512 particles of block bi (held
//   in registers, two per f32x2 lane pair), the records of block bj stream
//   through shared memory in tiles (bulk copies). Within a warp the 32
//   records of a group are visited in a rotation: at step k lane l pairs its
//   four particles with record (l + k) mod 32, whose running sums travel
//   with it from lane to lane by shuffles and are back at their home lane
//   after 32 steps. The four warps' sums per record are added in warp order
//   in shared memory and added into the workspace slot (bi, record). The bi
//   particles' own sums are folded per tile into compensated (hi, lo) pairs
//   and written to slot (bj, particle) after the pass.
// * Item (b, b): every ordered pair of the block, into slot (b, particle),
//   by the operation's own CTA body or by the rotation from the particle
//   side only.
// * Every particle thus has exactly nb slot partials (one per partner
//   block); a finalize kernel adds them in block order in FP64 and applies
//   the output transforms. The result does not depend on scheduling.
//
// Every wait on a tile is bounded (tile_stream.cuh).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>

#include "nbody.h"
#include "plan.cuh"
#include "regfuncs.cuh"
#include "tile_stream.cuh"

namespace cvtx {
namespace {

constexpr int kSymNT = 128;                    // threads per CTA
constexpr int kSymTPT = 4;                     // particles per thread and pass
constexpr int kSymH = kSymTPT / 2;             // f32x2 lane pairs per thread
constexpr int kSymPass = kSymNT * kSymTPT;     // particles of block bi per pass
constexpr int kSymWarps = kSymNT / 32;

// ---- pair operations -------------------------------------------------------
// An operation supplies: Problem (with src, n_tgt) and Consts; NC sums per
// particle; kRec float4 per record and kTile records per streamed tile;
// kMinBlocks, the resident CTAs per SM its registers are sized for;
// kUnroll, the rotation steps unrolled; kPlanFactor, the block plan's
// factor (sym_plan); the per-lane particle data (Tgt:
// four particles as two f32x2 lane pairs) and its loader (indices clamped
// below `lim`); step<FULL, SYM>, one lane's particles against one record in
// shared memory, adding to the particles' packed sums `acc` and (SYM) to the
// record's running sums `js` (FULL = false zeroes the pair for a lane whose
// record lies past the end of the block, `valid` false); write, the output
// of a particle from its FP64 sums; kOwnDiagonal and, if set, diagonal(),
// the CTA body for a diagonal item.

// ---- the rotation ------------------------------------------------------------
template <class Op> using SymStream = TileStream<Op::kRec, Op::kTile, 2>;

template <class Op>
constexpr size_t sym_smem_bytes() {
	// tile stages, (hi, lo) per pass particle and sum, and two buffers of
	// per-warp record sums [2][warps][NC][32]
	return SymStream<Op>::kSmemBytes + size_t(2) * Op::NC * kSymPass * sizeof(float) +
		size_t(2) * kSymWarps * Op::NC * 32 * sizeof(float);
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
		Op::template step<FULL, SYM>(kc, grp + Op::kRec * jl, jl < gcnt, g, acc, js);
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
	using Stream = SymStream<Op>;
	float* hi = reinterpret_cast<float*>(smem + Stream::kSmemBytes);
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
				const float4* grp = st + Op::kRec * 32 * gi;
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
		if (!Stream::run_continue(smem, p.src, j0, nj, err, tcount, tile_fn)) return false;
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

// A diagonal item: the operation's own CTA body, or the rotation from the
// particle side only.
template <class Op>
__device__ __forceinline__ bool sym_diagonal(const typename Op::Problem& p,
	const typename Op::Consts& kc, const SymArgs& a, int b, unsigned char* smem, unsigned* err,
	unsigned& tcount)
{
	if constexpr (Op::kOwnDiagonal) return Op::diagonal(p, kc, a, b, smem, err, tcount);
	else return sym_item<Op, false>(p, kc, a, b, b, smem, err, tcount);
}

template <class Op>
__global__ void __launch_bounds__(kSymNT, Op::kMinBlocks)
sym_kernel(const typename Op::Problem p, const typename Op::Consts kc, const SymArgs a,
	int n_items, unsigned* next, unsigned* err)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__shared__ int item_s;
	if (blockDim.x != kSymNT) {
		if (threadIdx.x == 0) atomicOr(err, kErrBadLaunch);
		return;
	}
	if (!SymStream<Op>::init(smem, err)) return;
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
			? sym_diagonal<Op>(p, kc, a, bi, smem, err, tcount)
			: sym_item<Op, true>(p, kc, a, bi, bj, smem, err, tcount);
		if (!ok) return;
	}
}

// Sum of every particle's nb slot partials in block order (FP64), then the
// output transforms.
template <class Op>
__global__ void sym_finalize(const typename Op::Problem p, const typename Op::Consts kc,
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
	static const int occ = resident_ctas(sym_kernel<Op>, kSymNT, sym_smem_bytes<Op>());
	return occ;
}

// Block plan: nb about sqrt(Op::kPlanFactor x resident CTAs) blocks, so
// kPlanFactor / 2 items per resident CTA (so that the last items leave
// little of the GPU idle: a greedy schedule of the 1M-particle fused call
// keeps 98.9 % of the CTAs busy to the end with 26 against 97.5 % with 16;
// timed 970.4 against 968.4 G/s fused, 1,594 against 1,563 stretching
// alone), blocks a multiple of the 512-particle pass, and a workspace within
// `ws_cap` bytes (fewer, longer blocks otherwise).
struct SymPlan {
	int S = 0, nb = 0, n_items = 0;
	size_t slots_bytes = 0, counter_off = 0, ws_bytes = 0;
};

SymPlan sym_plan(int n, int nc, int capacity, size_t ws_cap, double factor) {
	SymPlan pl;
	int nb = int(std::ceil(std::sqrt(factor * capacity)));
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
// grow as blocks x particles: 1M particles, fused: 3.9 GB; 4M: 15.7 GB).
// CVTX_GB300_SYM_WS_CAP (bytes) lowers it, e.g. to test the fallback.
size_t sym_ws_cap() {
	static const size_t cap = [] {
		const char* e = std::getenv("CVTX_GB300_SYM_WS_CAP");
		const long long v = (e && *e) ? std::atoll(e) : 0;
		return v > 0 ? size_t(v) : size_t(16) << 30;
	}();
	return cap;
}

// The workspace of the form, or SIZE_MAX where the cap leaves fewer than two
// items per resident CTA (blocks so long that the GPU would idle; the
// ordered-pair kernels then serve the call).
template <class Op>
size_t sym_ws_bytes(int n, int num_sms, size_t ws_cap) {
	const int capacity = num_sms * sym_occupancy<Op>();
	const SymPlan pl = sym_plan(n, Op::NC, capacity, ws_cap ? ws_cap : sym_ws_cap(),
		Op::kPlanFactor);
	return pl.n_items < 2 * capacity ? SIZE_MAX : pl.ws_bytes;
}

template <class Op>
cudaError_t sym_launch(const typename Op::Problem& p, const typename Op::Consts& kc,
	const LaunchEnv& env)
{
	const int occ = sym_occupancy<Op>();
	const SymPlan pl = sym_plan(p.n_tgt, Op::NC, env.num_sms * occ,
		env.cap_to_ws ? env.ws_bytes : std::min(env.ws_bytes, sym_ws_cap()), Op::kPlanFactor);
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
	sym_kernel<Op><<<grid, kSymNT, sym_smem_bytes<Op>(), env.stream>>>(
		p, kc, a, pl.n_items, d_next, env.err);
	count_launch();
	sym_finalize<Op><<<(p.n_tgt + 255) / 256, 256, 0, env.stream>>>(p, kc, a.slots, pl.nb);
	count_launch();
	return cudaGetLastError();
}

// Smallest particle count that takes the self-interaction form
// (CVTX_GB300_SYM_MIN; 0 switches the form off). Below about 22,000 P3D
// particles the rule of two items per resident CTA keeps the ordered-pair
// kernels anyway; from there the form was timed faster on a GB300 (24,000 -
// 32,000 particles: stretching 1.54-1.64x, velocity 1.07-1.11x, fused up to
// 1.11x; P2D at 32,000: 1.49-1.65x).
int sym_min_particles() {
	static const int min_n = [] {
		const char* e = std::getenv("CVTX_GB300_SYM_MIN");
		return (e && *e) ? std::atoi(e) : 16384;
	}();
	return min_n;
}

bool sym_size_ok(int n) {
	const int min_n = sym_min_particles();
	return min_n > 0 && n >= min_n && n >= 2 * kSymPass;
}

}  // namespace
}  // namespace cvtx
