// batch.cu -- many independent P3D velocity / stretching problems of uneven
// size in one persistent launch, captured in a CUDA graph.
//
// A batch is cut into work items (problem, target block, source split). Items
// are sorted by cost (largest first) and claimed by persistent CTAs through an
// atomic counter, so small and large problems share the GPU without per-
// problem launches or tail effects. An item runs the same CTA body as the
// per-call kernel (p3d_induce.cuh). Problems with one split write results
// directly; otherwise each split writes FP64 partials and the CTA that
// completes a target block last (per-block arrival counter) adds that block's
// splits in split order and writes the results -- deterministic, independent
// of which CTA ran what. The counters reset themselves, so the captured graph
// can be replayed.
//
// The launch shape (targets per thread x threads per CTA) and the source chunk
// per item are chosen by a built-in autotuner (cvtx_gb300_batch_tune) that
// times every candidate on the batch itself.
//
// Problems whose targets are their own particles (tgt == src, stride 2, from
// 4,096 particles; CVTX_GB300_SYM_MIN overrides, 0 switches it off) run in
// the self-interaction form instead (p3d_sym_batch.h): a second persistent
// launch over the block-pair items of all of them, then one finalize launch;
// both are part of the captured graph.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cvortex/cvtx_gb300.h"
#include "p3d_induce.cuh"
#include "p3d_sym_batch.h"
#include "plan.cuh"
#include "runtime.h"

namespace cvtx {
namespace {

struct BatchProblem {
	P3DInduceProblem p;
	InduceConsts kc;
	double* partial;      // n_split * NC * n_tgt doubles (n_split > 1)
	unsigned* counters;   // one per target block (n_split > 1)
	int n_split;
	int src_per_split;
};

template <Reg R, bool VEL, bool DV, int TPT, int NT>
__global__ void __launch_bounds__(NT)
p3d_batch_kernel(const BatchProblem* __restrict__ probs, int n_probs,
	const int4* __restrict__ items, int n_items, unsigned* next, unsigned* err)
{
	constexpr int NC = InduceNC<VEL, DV>::value;
	extern __shared__ __align__(16) unsigned char smem[];
	__shared__ __align__(16) BatchProblem sp;
	__shared__ int s_item;
	__shared__ int s_last;
	if (__syncthreads_or(blockDim.x != NT)) {
		if (threadIdx.x == 0) atomicOr(err, kErrBadLaunch);
		return;
	}
	if (!P3DStream::init(smem, err)) return;
	unsigned tcount = 0;
	for (;;) {
		__syncthreads();
		if (threadIdx.x == 0) s_item = int(atomicAdd(next, 1u));
		__syncthreads();
		const int it = s_item;
		if (it >= n_items) break;
		const int4 w = items[it];
		if (w.x < 0 || w.x >= n_probs) {
			if (threadIdx.x == 0) atomicOr(err, kErrBadWork);
			continue;
		}
		if (threadIdx.x == 0) sp = probs[w.x];
		__syncthreads();
		if (w.y < 0 || w.y * (TPT * NT) >= sp.p.n_tgt || w.z < 0 || w.z >= sp.n_split) {
			if (threadIdx.x == 0) atomicOr(err, kErrBadWork);
			continue;
		}
		const int tbase = w.y * (TPT * NT);
		const int s_begin = w.z * sp.src_per_split;
		int n_s = sp.p.n_src - s_begin;
		n_s = n_s < sp.src_per_split ? n_s : sp.src_per_split;
		n_s = n_s > 0 ? n_s : 0;
		const bool ok = induce2_block<R, VEL, DV, TPT, NT>(sp.p, sp.kc, tbase, s_begin, n_s, smem,
			err, tcount, [&](int t, const double* acc) {
				if (sp.n_split == 1) {
					write_induce<VEL, DV>(sp.p, sp.kc, t, acc);
				} else {
#pragma unroll
					for (int c = 0; c < NC; ++c)
						sp.partial[(size_t(w.z) * NC + c) * sp.p.n_tgt + t] = acc[c];
				}
			});
		if (!ok) return;
		if (sp.n_split > 1) {
			__threadfence();
			__syncthreads();
			if (threadIdx.x == 0)
				s_last = atomicAdd(&sp.counters[w.y], 1u) == unsigned(sp.n_split - 1) ? 1 : 0;
			__syncthreads();
			if (s_last) {
				__threadfence();
#pragma unroll 1
				for (int k = 0; k < TPT; ++k) {
					const int t = tbase + k * NT + threadIdx.x;
					if (t >= sp.p.n_tgt) continue;
					double s[NC];
#pragma unroll
					for (int c = 0; c < NC; ++c) s[c] = 0.0;
					for (int q = 0; q < sp.n_split; ++q)
#pragma unroll
						for (int c = 0; c < NC; ++c)
							s[c] += __ldcg(&sp.partial[(size_t(q) * NC + c) * sp.p.n_tgt + t]);
					write_induce<VEL, DV>(sp.p, sp.kc, t, s);
				}
				if (threadIdx.x == 0) sp.counters[w.y] = 0u;
			}
		}
	}
}

// Candidate launch shapes of the persistent kernel (targets per thread,
// threads per CTA); all packed f32x2.
struct BatchShape { int tpt, nt; };
constexpr BatchShape kShapes[] = {{4, 128}, {2, 128}, {4, 64}};
constexpr int kNumShapes = 3;
constexpr int kChunks[] = {2048, 4096, 8192, 16384, 32768};
constexpr int kNumChunks = 5;

template <Reg R, bool VEL, bool DV, int TPT, int NT>
struct BatchVariant {
	static constexpr int NC = InduceNC<VEL, DV>::value;
	static constexpr size_t kSmem = induce_smem_bytes<TPT, NT, NC>();
	static auto fn() { return p3d_batch_kernel<R, VEL, DV, TPT, NT>; }
	static int occupancy() {
		static const int occ = resident_ctas(fn(), NT, kSmem);
		return occ;
	}
};

template <class F>
auto with_batch_variant(int reg, unsigned ops, int shape, F&& f) {
	auto by_shape = [&](auto rt, auto vt, auto dt) {
		constexpr Reg R = decltype(rt)::value;
		constexpr bool VEL = decltype(vt)::value, DV = decltype(dt)::value;
		switch (shape) {
		case 0: return f(BatchVariant<R, VEL, DV, 4, 128>{});
		case 1: return f(BatchVariant<R, VEL, DV, 2, 128>{});
		default: return f(BatchVariant<R, VEL, DV, 4, 64>{});
		}
	};
	auto by_ops = [&](auto rt) {
		switch (ops) {
		case kOpVel: return by_shape(rt, std::true_type{}, std::false_type{});
		case kOpDvort: return by_shape(rt, std::false_type{}, std::true_type{});
		default: return by_shape(rt, std::true_type{}, std::true_type{});
		}
	};
	switch (reg) {
	case 0: return by_ops(std::integral_constant<Reg, Reg::Singular>{});
	case 1: return by_ops(std::integral_constant<Reg, Reg::Winckelmans>{});
	case 2: return by_ops(std::integral_constant<Reg, Reg::Planetary>{});
	default: return by_ops(std::integral_constant<Reg, Reg::Gaussian>{});
	}
}

}  // namespace
}  // namespace cvtx

using namespace cvtx;

struct cvtx_gb300_batch {
	std::vector<cvtx_gb300_p3d_problem> in;
	int reg = 1;
	unsigned ops = 3;
	int device = 0;
	int num_sms = 0;
	// current plan
	int shape = 0, chunk = 8192, n_items = 0, grid = 0;
	size_t n_counters = 1;          // per-target-block arrival counters in use
	size_t smem = 0;
	DevBuf d_probs, d_items, d_partial, d_counters, d_next, d_err;
	// the self-interaction part
	std::vector<char> in_sym;       // per problem: served by the self part
	int n_sym_probs = 0, n_sym_items = 0, sym_grid = 0, sym_total = 0;
	size_t sym_slot_bytes = 0;
	DevBuf d_sprobs, d_sitems, d_sprefix, d_slots, d_snext;
	cudaStream_t stream = nullptr;
	cudaEvent_t ev_in = nullptr, ev_out = nullptr;
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	double pairs = 0.0;
	std::string error;
};

namespace {

int fail(cvtx_gb300_batch* b, const std::string& msg, int code) {
	b->error = msg;
	set_error("cvtx_gb300_batch: " + msg);
	return code;
}

void drop_graph(cvtx_gb300_batch* b) {
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->graph) cudaGraphDestroy(b->graph);
	b->exec = nullptr;
	b->graph = nullptr;
}

// Cut the batch into items for (shape, chunk) and upload the tables.
int plan_batch(cvtx_gb300_batch* b, int shape, int chunk) {
	const int tpt = kShapes[shape].tpt, nt = kShapes[shape].nt;
	const int per_block = tpt * nt;
	const int nc = (b->ops & kOpVel ? 3 : 0) + (b->ops & kOpDvort ? 6 : 0);
	std::vector<BatchProblem> probs(b->in.size());
	struct Item { int4 w; double cost; };
	std::vector<Item> items;
	size_t partial_doubles = 0, counters = 0;
	std::vector<size_t> part_off(b->in.size()), cnt_off(b->in.size());
	for (size_t i = 0; i < b->in.size(); ++i) {
		const cvtx_gb300_p3d_problem& q = b->in[i];
		BatchProblem& bp = probs[i];
		std::memset(&bp, 0, sizeof bp);
		bp.p.src = static_cast<const float4*>(q.src); bp.p.n_src = q.n_src;
		bp.p.tgt = static_cast<const float4*>(q.tgt); bp.p.tstride = q.tgt_stride;
		bp.p.n_tgt = q.n_tgt;
		bp.p.out_vel = (b->ops & kOpVel) ? q.vel_out : nullptr;
		bp.p.out_dvort = (b->ops & kOpDvort) ? q.dvort_out : nullptr;
		bp.p.sigma = q.sigma;
		bp.kc = make_induce_consts(b->reg, q.sigma);
		if (b->in_sym[i]) continue;      // served by the self-interaction part
		const int n_split = q.n_src > 0 ? std::max(1, (q.n_src + chunk - 1) / chunk) : 1;
		int per = q.n_src > 0 ? (q.n_src + n_split - 1) / n_split : kP3DTile;
		per = ((per + kP3DTile - 1) / kP3DTile) * kP3DTile;
		bp.n_split = n_split;
		bp.src_per_split = per;
		const int n_tb = (q.n_tgt + per_block - 1) / per_block;
		if (n_split > 1) {
			part_off[i] = partial_doubles;
			cnt_off[i] = counters;
			partial_doubles += size_t(n_split) * nc * size_t(q.n_tgt);
			counters += size_t(n_tb);
		}
		for (int tb = 0; tb < n_tb; ++tb)
			for (int sp = 0; sp < n_split; ++sp) {
				const int tg = std::min(per_block, q.n_tgt - tb * per_block);
				const int sc = std::min(per, q.n_src - sp * per);
				items.push_back({make_int4(int(i), tb, sp, 0), double(tg) * double(std::max(sc, 0))});
			}
	}
	std::stable_sort(items.begin(), items.end(),
		[](const Item& a, const Item& c) { return a.cost > c.cost; });
	cudaError_t e = b->d_partial.ensure(std::max<size_t>(partial_doubles, 1) * sizeof(double));
	if (e == cudaSuccess) e = b->d_counters.ensure(std::max<size_t>(counters, 1) * sizeof(unsigned));
	if (e == cudaSuccess) e = b->d_probs.ensure(probs.size() * sizeof(BatchProblem));
	if (e == cudaSuccess) e = b->d_items.ensure(std::max<size_t>(items.size(), 1) * sizeof(int4));
	if (e != cudaSuccess) return fail(b, std::string("allocation: ") + cudaGetErrorString(e), -2);
	for (size_t i = 0; i < probs.size(); ++i) {
		if (probs[i].n_split > 1) {
			probs[i].partial = static_cast<double*>(b->d_partial.ptr) + part_off[i];
			probs[i].counters = static_cast<unsigned*>(b->d_counters.ptr) + cnt_off[i];
		}
	}
	std::vector<int4> w(items.size());
	for (size_t i = 0; i < items.size(); ++i) w[i] = items[i].w;
	e = cudaMemcpy(b->d_probs.ptr, probs.data(), probs.size() * sizeof(BatchProblem),
		cudaMemcpyHostToDevice);
	if (e == cudaSuccess && !w.empty())
		e = cudaMemcpy(b->d_items.ptr, w.data(), w.size() * sizeof(int4), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(b->d_counters.ptr, 0, std::max<size_t>(counters, 1) * sizeof(unsigned));
	if (e != cudaSuccess) return fail(b, std::string("upload: ") + cudaGetErrorString(e), -2);
	b->shape = shape;
	b->chunk = chunk;
	b->n_items = int(items.size());
	b->n_counters = std::max<size_t>(counters, 1);
	with_batch_variant(b->reg, b->ops, shape, [&](auto var) {
		using V = decltype(var);
		b->smem = V::kSmem;
		b->grid = std::max(1, std::min(b->n_items, b->num_sms * V::occupancy()));
		return 0;
	});
	drop_graph(b);
	return 0;
}

// Smallest problem of the self-interaction part (0: none).
int batch_sym_min() {
	static const int v = [] {
		const char* e = std::getenv("CVTX_GB300_SYM_MIN");
		return (e && *e) ? std::atoi(e) : 4096;
	}();
	return v;
}

// Slot memory the self-interaction part may hold; problems beyond it (in
// input order) stay with the ordered-pair items.
constexpr size_t kBatchSymSlotCap = size_t(8) << 30;

// Select the problems of the self-interaction part, cut each into at most 16
// blocks (a multiple of 512 particles), list their block-pair items largest
// first and upload the tables. Independent of the ordered part's plan. If
// the tables cannot be allocated, every problem stays with the ordered part.
int plan_sym(cvtx_gb300_batch* b) {
	const int nc = (b->ops & kOpVel ? 3 : 0) + (b->ops & kOpDvort ? 6 : 0);
	const int min_n = batch_sym_min();
	b->in_sym.assign(b->in.size(), 0);
	std::vector<SymBatchProblem> probs;
	std::vector<size_t> slot_off;
	std::vector<int> prefix;
	struct Item { int4 w; double cost; };
	std::vector<Item> items;
	size_t slot_floats = 0;
	long long total = 0;
	for (size_t i = 0; i < b->in.size(); ++i) {
		const cvtx_gb300_p3d_problem& q = b->in[i];
		const int n = q.n_tgt;
		if (min_n <= 0 || n < min_n || n < 1024 || q.tgt != q.src || q.tgt_stride != 2 ||
			q.n_src != n)
			continue;
		const int nb_t = std::min(16, (n + 511) / 512);
		const int S = 512 * ((n + 512 * nb_t - 1) / (512 * nb_t));
		const int nb = (n + S - 1) / S;
		const size_t floats = (size_t(nb) * nc * size_t(n) + 63) & ~size_t(63);
		if ((slot_floats + floats) * sizeof(float) > kBatchSymSlotCap) continue;
		b->in_sym[i] = 1;
		SymBatchProblem r;
		std::memset(&r, 0, sizeof r);
		r.p.src = static_cast<const float4*>(q.src); r.p.n_src = n;
		r.p.tgt = static_cast<const float4*>(q.src); r.p.tstride = 2; r.p.n_tgt = n;
		r.p.out_vel = (b->ops & kOpVel) ? q.vel_out : nullptr;
		r.p.out_dvort = (b->ops & kOpDvort) ? q.dvort_out : nullptr;
		r.p.sigma = q.sigma;
		r.kc = make_induce_consts(b->reg, q.sigma);
		r.S = S;
		r.nb = nb;
		const int k = int(probs.size());
		probs.push_back(r);
		slot_off.push_back(slot_floats);
		slot_floats += floats;
		prefix.push_back(int(total));
		total += n;
		for (int bj = 0; bj < nb; ++bj)
			for (int bi = 0; bi <= bj; ++bi) {
				const double li = std::min(S, n - bi * S), lj = std::min(S, n - bj * S);
				items.push_back({make_int4(k, bi, bj, 0), li * lj * (bi == bj ? 0.5 : 1.0)});
			}
	}
	b->n_sym_probs = int(probs.size());
	b->n_sym_items = int(items.size());
	if (probs.empty()) return 0;
	if (total > (long long)(1 << 30)) return fail(b, "self-interaction part too large", -1);
	prefix.push_back(int(total));
	b->sym_total = int(total);
	std::stable_sort(items.begin(), items.end(),
		[](const Item& a, const Item& c) { return a.cost > c.cost; });
	b->sym_slot_bytes = slot_floats * sizeof(float);
	cudaError_t e = b->d_slots.ensure(b->sym_slot_bytes);
	if (e == cudaSuccess) e = b->d_sprobs.ensure(probs.size() * sizeof(SymBatchProblem));
	if (e == cudaSuccess) e = b->d_sitems.ensure(items.size() * sizeof(int4));
	if (e == cudaSuccess) e = b->d_sprefix.ensure(prefix.size() * sizeof(int));
	if (e == cudaSuccess) e = b->d_snext.ensure(sizeof(unsigned));
	if (e == cudaErrorMemoryAllocation) {
		// no room for the tables: the ordered part serves every problem
		(void)cudaGetLastError();
		b->in_sym.assign(b->in.size(), 0);
		b->n_sym_probs = b->n_sym_items = 0;
		b->d_slots.release();
		return 0;
	}
	if (e != cudaSuccess) return fail(b, std::string("allocation: ") + cudaGetErrorString(e), -2);
	for (size_t k = 0; k < probs.size(); ++k)
		probs[k].slots = static_cast<float*>(b->d_slots.ptr) + slot_off[k];
	std::vector<int4> w(items.size());
	for (size_t i = 0; i < items.size(); ++i) w[i] = items[i].w;
	e = cudaMemcpy(b->d_sprobs.ptr, probs.data(), probs.size() * sizeof(SymBatchProblem),
		cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMemcpy(b->d_sitems.ptr, w.data(), w.size() * sizeof(int4), cudaMemcpyHostToDevice);
	if (e == cudaSuccess)
		e = cudaMemcpy(b->d_sprefix.ptr, prefix.data(), prefix.size() * sizeof(int),
			cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return fail(b, std::string("upload: ") + cudaGetErrorString(e), -2);
	b->sym_grid = std::max(1, std::min(b->n_sym_items,
		b->num_sms * p3d_sym_batch_occupancy(b->reg, b->ops)));
	return 0;
}

// Enqueue one batch execution on the batch's stream (not via the graph).
cudaError_t enqueue(cvtx_gb300_batch* b) {
	cudaError_t e = cudaSuccess;
	if (b->n_items > 0) {
		e = cudaMemsetAsync(b->d_next.ptr, 0, sizeof(unsigned), b->stream);
		if (e != cudaSuccess) return e;
		with_batch_variant(b->reg, b->ops, b->shape, [&](auto var) {
			using V = decltype(var);
			V::fn()<<<b->grid, kShapes[b->shape].nt, b->smem, b->stream>>>(
				static_cast<const BatchProblem*>(b->d_probs.ptr), int(b->in.size()),
				static_cast<const int4*>(b->d_items.ptr), b->n_items, static_cast<unsigned*>(b->d_next.ptr), static_cast<unsigned*>(b->d_err.ptr));
			return 0;
		});
		count_launch();
		e = cudaGetLastError();
		if (e != cudaSuccess) return e;
	}
	if (b->n_sym_items > 0) {
		// the slots and the item counter start at zero
		e = cudaMemsetAsync(b->d_slots.ptr, 0, b->sym_slot_bytes, b->stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(b->d_snext.ptr, 0, sizeof(unsigned), b->stream);
		if (e == cudaSuccess)
			e = p3d_sym_batch_enqueue(b->reg, b->ops,
				static_cast<const SymBatchProblem*>(b->d_sprobs.ptr), b->n_sym_probs,
				static_cast<const int4*>(b->d_sitems.ptr), b->n_sym_items,
				static_cast<const int*>(b->d_sprefix.ptr), b->sym_total,
				static_cast<unsigned*>(b->d_snext.ptr), static_cast<unsigned*>(b->d_err.ptr),
				b->sym_grid, b->stream);
	}
	return e;
}

// A CTA whose wait expired returns before it counts its arrival at its
// target block, so after a reported error the arrival counters are reset
// too: otherwise a later run could take a block's last arrival for complete
// before every split had written its partials.
int check_err_word(cvtx_gb300_batch* b) {
	unsigned w = 0;
	if (cudaMemcpy(&w, b->d_err.ptr, sizeof w, cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
	if (w) {
		cudaMemset(b->d_err.ptr, 0, sizeof w);
		cudaMemset(b->d_counters.ptr, 0, b->n_counters * sizeof(unsigned));
		return fail(b, device_error_text(w), -4);
	}
	return 0;
}

}  // namespace

extern "C" {

CVTX_EXPORT cvtx_gb300_batch* cvtx_gb300_batch_create(const cvtx_gb300_p3d_problem* problems,
	int n_problems, int reg, int ops)
{
	if (!problems || n_problems < 0 || reg < 0 || reg > 3 || ops < 1 || ops > 3) return nullptr;
	for (int i = 0; i < n_problems; ++i) {
		const cvtx_gb300_p3d_problem& q = problems[i];
		if (q.n_src < 0 || q.n_tgt < 0 || (q.n_tgt > 0 && !q.tgt) || (q.n_src > 0 && !q.src))
			return nullptr;
		if ((ops & 1) && q.n_tgt > 0 && !q.vel_out) return nullptr;
		if ((ops & 2) && q.n_tgt > 0 && (!q.dvort_out || q.tgt_stride < 2)) return nullptr;
		if (q.tgt_stride < 1) return nullptr;
	}
	auto* b = new cvtx_gb300_batch();
	b->in.assign(problems, problems + n_problems);
	b->reg = reg;
	b->ops = unsigned(ops);
	{
		std::lock_guard<std::recursive_mutex> g(Runtime::get().lock());
		DeviceContext* c = Runtime::get().active_context();
		if (!c) { delete b; set_error("cvtx_gb300_batch_create: no GPU enabled"); return nullptr; }
		b->device = c->device;
		b->num_sms = c->num_sms;
	}
	DeviceGuard dg(b->device);
	cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming);
	if (e == cudaSuccess) e = b->d_next.ensure(sizeof(unsigned));
	if (e == cudaSuccess) e = b->d_err.ensure(sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMemset(b->d_err.ptr, 0, sizeof(unsigned));
	if (e != cudaSuccess || plan_sym(b) != 0 || plan_batch(b, 0, 8192) != 0) {
		set_error(std::string("cvtx_gb300_batch_create: ") + cudaGetErrorString(e));
		cvtx_gb300_batch_destroy(b);
		return nullptr;
	}
	for (const auto& q : b->in) b->pairs += double(q.n_src) * double(q.n_tgt);
	return b;
}

// Time every (launch shape, source chunk) on this batch (`repeats` timed runs
// each, after one warm run) and keep the fastest.
CVTX_EXPORT int cvtx_gb300_batch_tune(cvtx_gb300_batch* b, int repeats) {
	if (!b || repeats < 1) return -1;
	DeviceGuard dg(b->device);
	cudaEvent_t t0, t1;
	cudaEventCreate(&t0);
	cudaEventCreate(&t1);
	float best = 1e30f;
	int best_shape = b->shape, best_chunk = b->chunk;
	for (int s = 0; s < kNumShapes; ++s) {
		for (int ci = 0; ci < kNumChunks; ++ci) {
			if (plan_batch(b, s, kChunks[ci]) != 0) continue;
			cudaError_t e = enqueue(b);
			cudaEventRecord(t0, b->stream);
			for (int r = 0; r < repeats && e == cudaSuccess; ++r) e = enqueue(b);
			cudaEventRecord(t1, b->stream);
			if (e == cudaSuccess) e = cudaEventSynchronize(t1);
			float ms = 0.f;
			if (e == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
			if (e != cudaSuccess) {
				cudaEventDestroy(t0); cudaEventDestroy(t1);
				return fail(b, std::string("tune: ") + cudaGetErrorString(e), -2);
			}
			if (ms < best) { best = ms; best_shape = s; best_chunk = kChunks[ci]; }
		}
	}
	cudaEventDestroy(t0);
	cudaEventDestroy(t1);
	if (plan_batch(b, best_shape, best_chunk) != 0) return -2;
	return check_err_word(b);
}

// Capture the current plan into a CUDA graph; later runs replay it.
CVTX_EXPORT int cvtx_gb300_batch_capture(cvtx_gb300_batch* b) {
	if (!b) return -1;
	DeviceGuard dg(b->device);
	drop_graph(b);
	cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
	if (e == cudaSuccess) {
		cudaError_t e2 = enqueue(b);
		e = cudaStreamEndCapture(b->stream, &b->graph);
		if (e == cudaSuccess) e = e2;
	}
	if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
	if (e != cudaSuccess) {
		drop_graph(b);
		return fail(b, std::string("capture: ") + cudaGetErrorString(e), -2);
	}
	return 0;
}

// Run the batch: ordered after earlier work on `stream` and before later work
// on it (the batch executes on its own stream in between).
CVTX_EXPORT int cvtx_gb300_batch_run(cvtx_gb300_batch* b, void* stream) {
	if (!b) return -1;
	DeviceGuard dg(b->device);
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	cudaError_t e = cudaEventRecord(b->ev_in, s);
	if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->ev_in, 0);
	if (e == cudaSuccess) {
		if (b->exec) {
			e = cudaGraphLaunch(b->exec, b->stream);
			count_launch();
		} else {
			e = enqueue(b);
		}
	}
	if (e == cudaSuccess) e = cudaEventRecord(b->ev_out, b->stream);
	if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->ev_out, 0);
	if (e != cudaSuccess) return fail(b, std::string("run: ") + cudaGetErrorString(e), -2);
	return 0;
}

// Synchronise and report a device-side timeout of earlier runs.
CVTX_EXPORT int cvtx_gb300_batch_status(cvtx_gb300_batch* b) {
	if (!b) return -1;
	DeviceGuard dg(b->device);
	if (cudaStreamSynchronize(b->stream) != cudaSuccess) return -2;
	return check_err_word(b);
}

CVTX_EXPORT int cvtx_gb300_batch_info(const cvtx_gb300_batch* b, int* shape_tpt,
	int* shape_nt, int* chunk, int* n_items, int* graph, double* interactions)
{
	if (!b) return -1;
	if (shape_tpt) *shape_tpt = kShapes[b->shape].tpt;
	if (shape_nt) *shape_nt = kShapes[b->shape].nt;
	if (chunk) *chunk = b->chunk;
	if (n_items) *n_items = b->n_items + b->n_sym_items;
	if (graph) *graph = b->exec ? 1 : 0;
	if (interactions) *interactions = b->pairs;
	return 0;
}

CVTX_EXPORT void cvtx_gb300_batch_destroy(cvtx_gb300_batch* b) {
	if (!b) return;
	DeviceGuard dg(b->device);
	if (b->stream) cudaStreamSynchronize(b->stream);
	drop_graph(b);
	b->d_probs.release(); b->d_items.release(); b->d_partial.release();
	b->d_counters.release(); b->d_next.release(); b->d_err.release();
	b->d_sprobs.release(); b->d_sitems.release(); b->d_sprefix.release();
	b->d_slots.release(); b->d_snext.release();
	if (b->ev_in) cudaEventDestroy(b->ev_in);
	if (b->ev_out) cudaEventDestroy(b->ev_out);
	if (b->stream) cudaStreamDestroy(b->stream);
	delete b;
}

}  // extern "C"
