// serve.cpp -- serving loop: continuous batching of M2M requests.
//
// The reference has no server: every cvtx_*_M2M call is a blocking,
// self-contained round trip (gather, upload, compute, download;
// src/P3D.cpp:343-366, src/ocl_P3D.cpp:150-321). Here requests of different
// kinds and sizes arrive from any thread and share one GPU:
//
//  * Admission. A scheduler thread takes requests in arrival order. A request
//    needs one slot (CUDA streams, a fixed split-sum workspace and an error
//    word) and one range of the device arena, a single
//    allocation made at start-up whose size is the HBM budget. While no slot
//    or no arena range is free the queue waits; it resumes as running
//    requests complete. A request larger than the whole budget is rejected.
//  * Resident state. An admitted request's state is uploaded once, advanced on
//    the device for all of its time steps (all-pairs M2M, then a forward-Euler
//    update) and downloaded once.
//  * Overlap. Every slot runs on its own streams, so requests admitted while
//    others are on the GPU run beside them. A slot has one stream per CUDA
//    stream priority level, and a request runs at a priority set by its
//    work per step (smaller = higher), so the block scheduler serves the CTAs
//    of small requests ahead of the waves of large ones. Running CTAs are
//    not preempted, so served launches bound the sources per CTA
//    (kCtaSrcCap) and a small request's kernel waits about 1 ms for SMs.
//    The default 32 slots match the hardware work queues at
//    CUDA_DEVICE_MAX_CONNECTIONS=32, which serving processes should set
//    before CUDA starts; the streams are created so that slots do not share
//    a queue.
//  * Determinism. A launch's source partition and reduction order depend only
//    on its problem size and the slot workspace size (equal for all slots),
//    never on what else is in flight, so a result is bit-identical alone and
//    in any mix.
//  * Completion. A host callback at the end of each slot's stream work hands
//    the slot back to the scheduler, which copies staged outputs into the
//    caller's memory, releases the arena ranges and records the latency.
//
// Host callbacks never call CUDA and the scheduler never holds its mutex
// while it calls CUDA, so a full stream cannot wait on a blocked callback.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cvortex/cvtx_gb300.h"
#include "nbody.h"
#include "runtime.h"

namespace cvtx {
namespace {

using Clock = std::chrono::steady_clock;
double now_s() {
	return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

constexpr size_t kAlign = 256;
// Split partials per slot. A 200,000-particle P3D step fits 37 splits
// (9 FP64 sums per target), about 5,400 sources per CTA.
constexpr size_t kSlotWsBytes = size_t(512) << 20;
// Sources per CTA in served launches (within the workspace): about 1 ms of
// FMA work per CTA for the fused P3D kernel, so a newly launched
// high-priority kernel waits about that long for SMs held by the CTAs of
// large requests. (8,192 gave p50 29-31 ms at 100 req/s and 68-81 ms at
// 300 req/s; 4,096 gives 24-25 and 55 ms, for 0.2 % of the throughput.)
constexpr int kCtaSrcCap = 4096;
constexpr size_t kStagingBytes = size_t(1) << 30;        // pinned staging arena
constexpr size_t kDefaultMaxHbm = size_t(64) << 30;
// One slot per hardware work queue at CUDA_DEVICE_MAX_CONNECTIONS=32.
constexpr int kDefaultSlots = 32;
constexpr int kMaxLevels = 8;                              // stream priority levels used
constexpr size_t kKeepFinished = size_t(1) << 20;          // finished records kept
inline size_t up(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }

// First-fit range allocator over [0, cap) with coalescing of free ranges.
class Arena {
 public:
	void reset(size_t cap) {
		cap_ = cap; used_ = peak_ = 0;
		free_.clear();
		if (cap) free_[0] = cap;
	}
	bool alloc(size_t bytes, size_t* off) {
		if (bytes == 0) { *off = 0; return true; }
		for (auto it = free_.begin(); it != free_.end(); ++it) {
			if (it->second < bytes) continue;
			*off = it->first;
			const size_t rest = it->second - bytes, next = it->first + bytes;
			free_.erase(it);
			if (rest) free_[next] = rest;
			used_ += bytes;
			peak_ = std::max(peak_, used_);
			return true;
		}
		return false;
	}
	void release(size_t off, size_t bytes) {
		if (bytes == 0) return;
		auto it = free_.emplace(off, bytes).first;
		auto nx = std::next(it);
		if (nx != free_.end() && it->first + it->second == nx->first) {
			it->second += nx->second;
			free_.erase(nx);
		}
		if (it != free_.begin()) {
			auto pv = std::prev(it);
			if (pv->first + pv->second == it->first) {
				pv->second += it->second;
				free_.erase(it);
			}
		}
		used_ -= bytes;
	}
	size_t cap() const { return cap_; }
	size_t used() const { return used_; }
	size_t peak() const { return peak_; }
	void reset_peak() { peak_ = used_; }

 private:
	size_t cap_ = 0, used_ = 0, peak_ = 0;
	std::map<size_t, size_t> free_;
};

// Byte sizes of a request's device buffers (each 256-byte aligned).
struct Layout {
	size_t state = 0, tgt = 0, vel = 0, dvort = 0;    // offsets
	size_t state_b = 0, tgt_b = 0, vel_b = 0, dvort_b = 0;
	size_t total = 0;
};
Layout layout_of(const cvtx_gb300_request& r) {
	Layout L;
	const size_t n = size_t(r.n);
	switch (r.kind) {
	case CVTX_GB300_REQ_P3D: L.state_b = 32 * n; L.vel_b = 12 * n; L.dvort_b = 12 * n; break;
	case CVTX_GB300_REQ_P2D: L.state_b = 16 * n; L.vel_b = 8 * n; break;
	default:
		L.state_b = 32 * n;
		L.tgt_b = 16 * size_t(r.n_tgt);
		L.vel_b = 12 * size_t(r.n_tgt);
		break;
	}
	size_t o = 0;
	L.state = o; o += up(L.state_b);
	L.tgt = o; o += up(L.tgt_b);
	L.vel = o; o += up(L.vel_b);
	L.dvort = o; o += up(L.dvort_b);
	L.total = o;
	return L;
}
// Bytes of the state written back (P3D / P2D particles, or F3D tracer points).
size_t out_state_bytes(const cvtx_gb300_request& r, const Layout& L) {
	return r.kind == CVTX_GB300_REQ_F3D ? L.tgt_b : L.state_b;
}
double pairs_of(const cvtx_gb300_request& r) {
	const double tg = r.kind == CVTX_GB300_REQ_F3D ? double(r.n_tgt) : double(r.n);
	return double(r.n) * tg * double(r.n_steps);
}

bool valid(const cvtx_gb300_request* r) {
	if (!r) return false;
	if (r->kind < CVTX_GB300_REQ_P3D || r->kind > CVTX_GB300_REQ_F3D) return false;
	if (r->n < 1 || r->n > (1 << 26) || r->n_steps < 1 || r->n_steps > (1 << 24)) return false;
	if (!std::isfinite(r->dt) || !r->state_in || !r->state_out) return false;
	if (r->kind == CVTX_GB300_REQ_F3D) {
		if (r->n_tgt < 1 || r->n_tgt > (1 << 26) || !r->tgt_in) return false;
	} else {
		if (r->reg < 0 || r->reg > 3 || !std::isfinite(r->sigma)) return false;
	}
	return true;
}

// Page-locked (cudaHostAlloc / registered) host memory can be the direct
// source or target of an asynchronous copy; anything else is staged.
bool is_pinned(const void* p) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeHost;
}

struct Request {
	cvtx_gb300_request r{};
	unsigned long long id = 0;
	int status = CVTX_GB300_ST_PENDING;
	double t_submit = 0, t_admit = 0, t_done = 0;
	Layout L;
	size_t dev_off = 0;
	int slot = -1;
	// pinned staging: offsets into the staging arena, or SIZE_MAX when the
	// caller's buffer is used directly
	size_t host_off = 0, host_bytes = 0;
	size_t st_in = SIZE_MAX, st_tgt = SIZE_MAX, st_out = SIZE_MAX, st_vel = SIZE_MAX;
};

class Server;
struct Slot {
	Server* srv = nullptr;
	int index = 0;
	cudaStream_t st[kMaxLevels] = {};   // one stream per priority level, highest first
	void* ws = nullptr;
	unsigned* d_err = nullptr;
	unsigned* h_err = nullptr;      // pinned
	unsigned long long req = 0;
	cudaError_t launch_error = cudaSuccess;
};

class Server {
 public:
	~Server() { shutdown(); }

	bool open(int n_slots, size_t hbm, bool dry, std::string* why);
	unsigned long long submit(const cvtx_gb300_request* r);
	int wait(unsigned long long id, double timeout_ms);
	int drain(double timeout_ms);
	int info(unsigned long long id, double* lat, double* q);
	void stats(cvtx_gb300_server_stats* out);
	void reset_stats();
	void inject(int n) {
		std::lock_guard<std::mutex> g(mu_);
		inject_ += n > 0 ? n : 0;
	}
	void shutdown();

	// host callback (a CUDA driver thread): no CUDA calls in here
	void gpu_done(int slot) {
		{
			std::lock_guard<std::mutex> g(mu_);
			done_slots_.push_back(slot);
		}
		cv_.notify_all();
	}

 private:
	void loop();
	void admit(std::unique_lock<std::mutex>& lk);
	void finish(int s, std::unique_lock<std::mutex>& lk);
	void complete_locked(Request& q, int status);
	cudaError_t launch(Request& q, Slot& sl);
	cudaError_t warm_up();
	bool can_admit() const {
		return !queue_.empty() && !free_slots_.empty() && !mem_blocked_;
	}

	// Priority level of a request: the highest for under 2^24 pairs per step,
	// one level lower for every further factor of 16 (shortest work first at
	// the block scheduler, without reordering the admission queue).
	int level_of(double pairs_per_step) const {
		int l = 0;
		double lim = double(1 << 24);
		while (l + 1 < levels_ && pairs_per_step >= lim) { ++l; lim *= 16.0; }
		return l;
	}

	bool dry_ = false;
	int levels_ = 1;
	int device_ = 0, num_sms_ = 1;
	void* d_arena_ = nullptr;
	unsigned char* h_stage_ = nullptr;
	std::vector<Slot> slots_;

	std::mutex mu_;
	std::condition_variable cv_;        // scheduler wake-up
	std::condition_variable done_cv_;   // request completion
	bool stop_ = false;
	std::thread thread_;
	Arena dev_, host_;
	// shared so that a waiter keeps its record alive when it is forgotten
	std::unordered_map<unsigned long long, std::shared_ptr<Request>> reqs_;
	std::deque<unsigned long long> finished_;   // oldest first
	std::deque<unsigned long long> queue_;
	std::vector<int> free_slots_;
	std::deque<int> done_slots_;
	unsigned long long next_id_ = 1;
	int inflight_ = 0;
	bool mem_blocked_ = false;
	int inject_ = 0;

	// statistics since the last reset
	unsigned long long submitted_ = 0, completed_ = 0, rejected_ = 0, failed_ = 0;
	std::vector<double> lat_ms_, queue_ms_;
	double interactions_ = 0, first_submit_ = 0, last_done_ = 0;
	unsigned long long launches0_ = 0;
};

void CUDART_CB on_slot_done(void* p) {
	auto* s = static_cast<Slot*>(p);
	s->srv->gpu_done(s->index);
}

bool Server::open(int n_slots, size_t hbm, bool dry, std::string* why) {
	dry_ = dry;
	if (n_slots <= 0) n_slots = kDefaultSlots;
	if (n_slots > 256) n_slots = 256;
	slots_.resize(size_t(n_slots));
	if (!dry_) {
		{
			auto& rt = Runtime::get();
			std::lock_guard<std::recursive_mutex> g(rt.lock());
			DeviceContext* ctx = rt.active_context();
			if (!ctx) { *why = "no enabled CUDA accelerator"; return false; }
			device_ = ctx->device;
			num_sms_ = ctx->num_sms;
		}
		cudaError_t e = cudaSetDevice(device_);
		size_t free_b = 0, total_b = 0;
		if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
		if (e != cudaSuccess) { *why = cudaGetErrorString(e); return false; }
		if (hbm == 0) hbm = std::min(free_b / 2, kDefaultMaxHbm);
		hbm &= ~(kAlign - 1);
		const size_t fixed = size_t(n_slots) * kSlotWsBytes;
		if (hbm + fixed > free_b) { *why = "HBM budget exceeds free device memory"; return false; }
		e = cudaMalloc(&d_arena_, hbm);
		if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&h_stage_), kStagingBytes,
			cudaHostAllocDefault);
		int lo_pri = 0, hi_pri = 0;
		if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri);
		// numerically lower = higher priority; hi_pri <= lo_pri
		levels_ = std::min(kMaxLevels, lo_pri - hi_pri + 1);
		if (levels_ < 1) levels_ = 1;
		// Streams are created level by level, slot by slot. CUDA maps streams
		// onto its hardware work queues in creation order, so with n_slots
		// equal to the queue count (CUDA_DEVICE_MAX_CONNECTIONS) a slot's
		// streams of every level share one queue and no two slots share one:
		// a request never waits in a queue behind another request's kernels.
		for (int l = 0; e == cudaSuccess && l < levels_; ++l)
			for (int i = 0; e == cudaSuccess && i < n_slots; ++i)
				e = cudaStreamCreateWithPriority(&slots_[size_t(i)].st[l], cudaStreamNonBlocking,
					hi_pri + l);
		for (int i = 0; e == cudaSuccess && i < n_slots; ++i) {
			Slot& s = slots_[size_t(i)];
			if (e == cudaSuccess) e = cudaMalloc(&s.ws, kSlotWsBytes);
			if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&s.d_err), sizeof(unsigned));
			if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&s.h_err), sizeof(unsigned),
				cudaHostAllocDefault);
		}
		if (e != cudaSuccess) { *why = cudaGetErrorString(e); return false; }
	} else if (hbm == 0) {
		hbm = size_t(1) << 30;
	}
	dev_.reset(hbm);
	host_.reset(kStagingBytes);
	for (int i = 0; i < n_slots; ++i) {
		slots_[size_t(i)].srv = this;
		slots_[size_t(i)].index = i;
		free_slots_.push_back(n_slots - 1 - i);
	}
	if (!dry_) {
		const cudaError_t e = warm_up();
		if (e != cudaSuccess) { *why = cudaGetErrorString(e); return false; }
	}
	launches0_ = launch_count();
	thread_ = std::thread([this] { loop(); });
	return true;
}

// Every kernel a served request can launch, launched once on zeroed scratch
// records through the same dispatch and launch environment as served
// requests, with sizes that reach every branch of the launch choice (the
// few-target form, configuration 0, mid-size and large packed forms) and
// every regularisation. CUDA loads a kernel's code at its first launch by
// default (lazy loading), and that load stalls other work on the device:
// without this the first requests to need a new kernel wait for everything
// in flight, about a second in a busy stream.
cudaError_t Server::warm_up() {
	const int p3d_n[] = {1, 8, 300, 9000, 40000};
	const int p2d_n[] = {1, 8, 3000, 9000, 70000};
	const int f3d_n[] = {1, 8, 3000, 9000};
	const size_t max_n = 70000;
	void* scratch = nullptr;
	cudaError_t e = cudaMalloc(&scratch, max_n * (32 + 16 + 12 + 12));
	if (e != cudaSuccess) return e;
	float4* rec = static_cast<float4*>(scratch);                  // 2 float4 per record
	float4* pts = rec + 2 * max_n;                                // 1 float4 per point
	float* out1 = reinterpret_cast<float*>(pts + max_n);          // 3 floats per target
	float* out2 = out1 + 3 * max_n;
	Slot& sl = slots_[0];
	cudaStream_t st = sl.st[0];
	e = cudaMemsetAsync(scratch, 0, max_n * (32 + 16 + 12 + 12), st);
	LaunchEnv env{sl.ws, kSlotWsBytes, sl.d_err, st, num_sms_, true, kCtaSrcCap};
	for (int reg = 0; e == cudaSuccess && reg < 4; ++reg) {
		for (int n : p3d_n) {
			if (e != cudaSuccess) break;
			P3DInduceProblem p;
			p.src = rec; p.n_src = n; p.tgt = rec; p.tstride = 2; p.n_tgt = n;
			p.out_vel = out1; p.out_dvort = out2; p.sigma = 0.05f;
			e = p3d_induce(reg, kOpVel | kOpDvort, p, env);
		}
		for (int n : p2d_n) {
			if (e != cudaSuccess) break;
			P2DVelProblem p;
			p.src = pts; p.n_src = n; p.tgt = pts; p.n_tgt = n; p.out = out1; p.sigma = 0.05f;
			e = p2d_vel(reg, p, env);
		}
	}
	for (int n : f3d_n) {
		if (e != cudaSuccess) break;
		F3DVelProblem p;
		p.fil = rec; p.n_fil = n; p.tgt = pts; p.tstride = 1; p.n_tgt = n; p.out = out1;
		e = f3d_vel(p, env);
	}
	if (e == cudaSuccess) e = advance_p3d(rec, 8, out1, out2, 0.f, st);
	if (e == cudaSuccess) e = advance_p2d(pts, 8, out1, 0.f, st);
	if (e == cudaSuccess) e = advance_points(pts, 8, out1, 0.f, st);
	if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_err, 0, sizeof(unsigned), st);
	const cudaError_t s = cudaStreamSynchronize(st);
	if (e == cudaSuccess) e = s;
	cudaFree(scratch);
	return e;
}

void Server::shutdown() {
	if (thread_.joinable()) {
		drain(-1.0);
		{
			std::lock_guard<std::mutex> g(mu_);
			stop_ = true;
		}
		cv_.notify_all();
		thread_.join();
	}
	if (!dry_) {
		for (Slot& s : slots_) {
			for (cudaStream_t q : s.st)
				if (q) {
					cudaStreamSynchronize(q);
					cudaStreamDestroy(q);
				}
			if (s.ws) cudaFree(s.ws);
			if (s.d_err) cudaFree(s.d_err);
			if (s.h_err) cudaFreeHost(s.h_err);
			s = Slot{};
		}
		if (d_arena_) cudaFree(d_arena_);
		if (h_stage_) cudaFreeHost(h_stage_);
		d_arena_ = nullptr;
		h_stage_ = nullptr;
	}
}

unsigned long long Server::submit(const cvtx_gb300_request* r) {
	if (!valid(r)) return 0;
	Request q;
	q.r = *r;
	q.L = layout_of(*r);
	// pageable caller buffers go through pinned staging
	const size_t in_b = q.L.state_b, out_b = out_state_bytes(*r, q.L);
	size_t h = 0;
	auto stage = [&](const void* p, size_t bytes, size_t* off) {
		if (!p || bytes == 0) return;
		if (!dry_ && is_pinned(p)) return;
		*off = h;
		h += up(bytes);
	};
	stage(r->state_in, in_b, &q.st_in);
	if (r->kind == CVTX_GB300_REQ_F3D) stage(r->tgt_in, q.L.tgt_b, &q.st_tgt);
	stage(r->state_out, out_b, &q.st_out);
	stage(r->vel_out, q.L.vel_b, &q.st_vel);
	q.host_bytes = h;
	unsigned long long id;
	{
		std::lock_guard<std::mutex> g(mu_);
		if (stop_) return 0;
		id = next_id_++;
		q.id = id;
		q.t_submit = now_s();
		if (submitted_ == 0) first_submit_ = q.t_submit;
		++submitted_;
		reqs_.emplace(id, std::make_shared<Request>(q));
		queue_.push_back(id);
	}
	cv_.notify_all();
	return id;
}

void Server::complete_locked(Request& q, int status) {
	q.status = status;
	q.t_done = now_s();
	last_done_ = q.t_done;
	if (status == CVTX_GB300_ST_DONE) {
		++completed_;
		lat_ms_.push_back(1e3 * (q.t_done - q.t_submit));
		queue_ms_.push_back(1e3 * (q.t_admit - q.t_submit));
		interactions_ += pairs_of(q.r);
	} else if (status == CVTX_GB300_ST_REJECTED || status == CVTX_GB300_ST_OOM) {
		++rejected_;
	} else {
		++failed_;
	}
	// keep a bounded number of finished records for wait / request_info
	finished_.push_back(q.id);
	if (finished_.size() > kKeepFinished) {
		reqs_.erase(finished_.front());
		finished_.pop_front();
	}
	done_cv_.notify_all();
}

void Server::loop() {
	if (!dry_) cudaSetDevice(device_);
	std::unique_lock<std::mutex> lk(mu_);
	for (;;) {
		cv_.wait(lk, [&] { return stop_ || !done_slots_.empty() || can_admit(); });
		while (!done_slots_.empty()) {
			const int s = done_slots_.front();
			done_slots_.pop_front();
			finish(s, lk);
		}
		admit(lk);
		if (stop_ && queue_.empty() && inflight_ == 0 && done_slots_.empty()) break;
	}
}

void Server::admit(std::unique_lock<std::mutex>& lk) {
	while (!queue_.empty() && !free_slots_.empty()) {
		Request& q = *reqs_.at(queue_.front());
		if (q.L.total > dev_.cap() || q.host_bytes > host_.cap()) {
			queue_.pop_front();
			complete_locked(q, CVTX_GB300_ST_REJECTED);
			continue;
		}
		const bool injected = inject_ > 0;
		if (injected) --inject_;
		size_t doff = 0, hoff = 0;
		bool ok = !injected && dev_.alloc(q.L.total, &doff);
		if (ok && !host_.alloc(q.host_bytes, &hoff)) {
			dev_.release(doff, q.L.total);
			ok = false;
		}
		if (!ok) {
			if (inflight_ == 0) {
				// nothing running will free memory: give up on this request
				queue_.pop_front();
				complete_locked(q, CVTX_GB300_ST_OOM);
				continue;
			}
			mem_blocked_ = true;    // retried after the next completion
			return;
		}
		queue_.pop_front();
		const int s = free_slots_.back();
		free_slots_.pop_back();
		q.dev_off = doff;
		q.host_off = hoff;
		q.slot = s;
		q.status = CVTX_GB300_ST_RUNNING;
		q.t_admit = now_s();
		++inflight_;
		Slot& sl = slots_[size_t(s)];
		sl.req = q.id;
		if (dry_) {
			done_slots_.push_back(s);
			continue;
		}
		// Launch without the lock: a launch may block on a full stream, which
		// may need a host callback (which takes the lock) to drain.
		lk.unlock();
		sl.launch_error = launch(q, sl);
		if (sl.launch_error != cudaSuccess) {
			for (cudaStream_t q : sl.st)
				if (q) cudaStreamSynchronize(q);
			cudaGetLastError();
		}
		lk.lock();
		if (sl.launch_error != cudaSuccess) done_slots_.push_back(s);
	}
}

cudaError_t Server::launch(Request& q, Slot& sl) {
	const cvtx_gb300_request& r = q.r;
	const Layout& L = q.L;
	cudaStream_t st = sl.st[level_of(pairs_of(r) / r.n_steps)];
	unsigned char* base = static_cast<unsigned char*>(d_arena_) + q.dev_off;
	float4* state = reinterpret_cast<float4*>(base + L.state);
	float4* tgt = reinterpret_cast<float4*>(base + L.tgt);
	float* vel = reinterpret_cast<float*>(base + L.vel);
	float* dvort = reinterpret_cast<float*>(base + L.dvort);
	unsigned char* hs = h_stage_ + q.host_off;
	auto src_of = [&](const float* user, size_t off, size_t bytes) -> const void* {
		if (off == SIZE_MAX) return user;
		std::memcpy(hs + off, user, bytes);
		return hs + off;
	};
	cudaError_t e = cudaMemsetAsync(sl.d_err, 0, sizeof(unsigned), st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(state, src_of(r.state_in, q.st_in, L.state_b), L.state_b,
			cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess && r.kind == CVTX_GB300_REQ_F3D)
		e = cudaMemcpyAsync(tgt, src_of(r.tgt_in, q.st_tgt, L.tgt_b), L.tgt_b,
			cudaMemcpyHostToDevice, st);
	LaunchEnv env{sl.ws, kSlotWsBytes, sl.d_err, st, num_sms_, true, kCtaSrcCap};
	for (int k = 0; e == cudaSuccess && k < r.n_steps; ++k) {
		switch (r.kind) {
		case CVTX_GB300_REQ_P3D: {
			P3DInduceProblem p;
			p.src = state; p.n_src = r.n;
			p.tgt = state; p.tstride = 2; p.n_tgt = r.n;
			p.out_vel = vel; p.out_dvort = dvort; p.sigma = r.sigma;
			e = p3d_induce(r.reg, kOpVel | kOpDvort, p, env);
			if (e == cudaSuccess) e = advance_p3d(state, r.n, vel, dvort, r.dt, st);
			break;
		}
		case CVTX_GB300_REQ_P2D: {
			P2DVelProblem p;
			p.src = state; p.n_src = r.n;
			p.tgt = state; p.n_tgt = r.n;
			p.out = vel; p.sigma = r.sigma;
			e = p2d_vel(r.reg, p, env);
			if (e == cudaSuccess) e = advance_p2d(state, r.n, vel, r.dt, st);
			break;
		}
		default: {
			F3DVelProblem p;
			p.fil = state; p.n_fil = r.n;
			p.tgt = tgt; p.tstride = 1; p.n_tgt = r.n_tgt;
			p.out = vel;
			e = f3d_vel(p, env);
			if (e == cudaSuccess) e = advance_points(tgt, r.n_tgt, vel, r.dt, st);
			break;
		}
		}
	}
	const size_t out_b = out_state_bytes(r, L);
	const void* dev_out = r.kind == CVTX_GB300_REQ_F3D ? static_cast<const void*>(tgt)
		: static_cast<const void*>(state);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(q.st_out == SIZE_MAX ? static_cast<void*>(r.state_out) : hs + q.st_out,
			dev_out, out_b, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess && r.vel_out)
		e = cudaMemcpyAsync(q.st_vel == SIZE_MAX ? static_cast<void*>(r.vel_out) : hs + q.st_vel,
			vel, L.vel_b, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(sl.h_err, sl.d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaLaunchHostFunc(st, on_slot_done, &sl);
	return e;
}

void Server::finish(int s, std::unique_lock<std::mutex>& lk) {
	Slot& sl = slots_[size_t(s)];
	Request& q = *reqs_.at(sl.req);
	int status = CVTX_GB300_ST_DONE;
	if (!dry_) {
		if (sl.launch_error != cudaSuccess) {
			status = CVTX_GB300_ST_FAILED;
			set_error(std::string("cvtx_gb300_server: ") + cudaGetErrorString(sl.launch_error));
		} else if (*sl.h_err != 0u) {
			status = CVTX_GB300_ST_TIMEOUT;
			set_error("cvtx_gb300_server: " + device_error_text(*sl.h_err));
		}
		if (status == CVTX_GB300_ST_DONE) {
			// staged outputs -> caller memory (outside the lock)
			lk.unlock();
			const unsigned char* hs = h_stage_ + q.host_off;
			if (q.st_out != SIZE_MAX)
				std::memcpy(q.r.state_out, hs + q.st_out, out_state_bytes(q.r, q.L));
			if (q.r.vel_out && q.st_vel != SIZE_MAX)
				std::memcpy(q.r.vel_out, hs + q.st_vel, q.L.vel_b);
			lk.lock();
		}
	}
	dev_.release(q.dev_off, q.L.total);
	host_.release(q.host_off, q.host_bytes);
	sl.req = 0;
	sl.launch_error = cudaSuccess;
	free_slots_.push_back(s);
	--inflight_;
	mem_blocked_ = false;
	complete_locked(q, status);
}

int Server::wait(unsigned long long id, double timeout_ms) {
	std::unique_lock<std::mutex> lk(mu_);
	auto it = reqs_.find(id);
	if (it == reqs_.end()) return CVTX_GB300_ST_UNKNOWN;
	const std::shared_ptr<Request> q = it->second;
	auto pred = [&] { return q->status <= CVTX_GB300_ST_DONE; };
	if (timeout_ms < 0) done_cv_.wait(lk, pred);
	else done_cv_.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), pred);
	return q->status;
}

int Server::drain(double timeout_ms) {
	std::unique_lock<std::mutex> lk(mu_);
	auto pred = [&] { return queue_.empty() && inflight_ == 0; };
	if (timeout_ms < 0) { done_cv_.wait(lk, pred); return 0; }
	return done_cv_.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), pred)
		? 0 : 1;
}

int Server::info(unsigned long long id, double* lat, double* qd) {
	std::lock_guard<std::mutex> g(mu_);
	auto it = reqs_.find(id);
	if (it == reqs_.end()) return CVTX_GB300_ST_UNKNOWN;
	const Request& q = *it->second;
	if (lat) *lat = q.status == CVTX_GB300_ST_DONE ? 1e3 * (q.t_done - q.t_submit) : -1.0;
	if (qd) *qd = q.t_admit > 0 ? 1e3 * (q.t_admit - q.t_submit) : -1.0;
	return q.status;
}

double pct(std::vector<double> v, double p) {
	if (v.empty()) return 0.0;
	// nearest-rank percentile
	size_t k = size_t(std::ceil(p * double(v.size()))) ;
	k = k == 0 ? 0 : k - 1;
	if (k >= v.size()) k = v.size() - 1;
	std::nth_element(v.begin(), v.begin() + std::ptrdiff_t(k), v.end());
	return v[k];
}

void Server::stats(cvtx_gb300_server_stats* o) {
	std::lock_guard<std::mutex> g(mu_);
	std::memset(o, 0, sizeof(*o));
	o->submitted = submitted_;
	o->completed = completed_;
	o->rejected = rejected_;
	o->failed = failed_;
	o->queued = queue_.size();
	o->in_flight = static_cast<unsigned long long>(inflight_);
	o->p50_ms = pct(lat_ms_, 0.50);
	o->p99_ms = pct(lat_ms_, 0.99);
	double sum = 0, mx = 0;
	for (double x : lat_ms_) { sum += x; mx = std::max(mx, x); }
	o->mean_ms = lat_ms_.empty() ? 0.0 : sum / double(lat_ms_.size());
	o->max_ms = mx;
	o->queue_p50_ms = pct(queue_ms_, 0.50);
	o->queue_p99_ms = pct(queue_ms_, 0.99);
	o->interactions = interactions_;
	o->span_s = last_done_ > first_submit_ ? last_done_ - first_submit_ : 0.0;
	o->hbm_budget = dev_.cap();
	o->hbm_used = dev_.used();
	o->hbm_peak = dev_.peak();
	o->kernel_launches = launch_count() - launches0_;
}

void Server::reset_stats() {
	std::lock_guard<std::mutex> g(mu_);
	submitted_ = completed_ = rejected_ = failed_ = 0;
	lat_ms_.clear();
	queue_ms_.clear();
	interactions_ = 0;
	first_submit_ = last_done_ = 0;
	dev_.reset_peak();
	launches0_ = launch_count();
	// forget finished requests
	finished_.clear();
	for (auto it = reqs_.begin(); it != reqs_.end();) {
		if (it->second->status <= CVTX_GB300_ST_DONE) it = reqs_.erase(it);
		else ++it;
	}
}

}  // namespace
}  // namespace cvtx

struct cvtx_gb300_server {
	cvtx::Server impl;
};

using namespace cvtx;

extern "C" {

CVTX_EXPORT cvtx_gb300_server* cvtx_gb300_server_create(int n_slots,
	unsigned long long hbm_bytes, int flags)
{
	auto* s = new cvtx_gb300_server();
	std::string why;
	if (!s->impl.open(n_slots, size_t(hbm_bytes), (flags & CVTX_GB300_SERVER_DRY_RUN) != 0, &why)) {
		set_error("cvtx_gb300_server_create: " + why);
		delete s;
		return nullptr;
	}
	return s;
}

CVTX_EXPORT unsigned long long cvtx_gb300_server_submit(cvtx_gb300_server* srv,
	const cvtx_gb300_request* req)
{
	if (!srv) return 0;
	return srv->impl.submit(req);
}

CVTX_EXPORT int cvtx_gb300_server_replay(cvtx_gb300_server* srv,
	const cvtx_gb300_request* reqs, const double* arrival_s, int n,
	unsigned long long* ids_out)
{
	if (!srv || n < 0 || (n > 0 && (!reqs || !arrival_s))) return -1;
	const auto t0 = Clock::now();
	for (int i = 0; i < n; ++i) {
		const auto at = t0 + std::chrono::duration_cast<Clock::duration>(
			std::chrono::duration<double>(arrival_s[i] > 0 ? arrival_s[i] : 0.0));
		std::this_thread::sleep_until(at);
		const unsigned long long id = srv->impl.submit(&reqs[i]);
		if (ids_out) ids_out[i] = id;
	}
	return 0;
}

CVTX_EXPORT int cvtx_gb300_server_wait(cvtx_gb300_server* srv, unsigned long long id,
	double timeout_ms)
{
	if (!srv) return CVTX_GB300_ST_UNKNOWN;
	return srv->impl.wait(id, timeout_ms);
}

CVTX_EXPORT int cvtx_gb300_server_drain(cvtx_gb300_server* srv, double timeout_ms) {
	if (!srv) return -1;
	return srv->impl.drain(timeout_ms);
}

CVTX_EXPORT int cvtx_gb300_server_request_info(cvtx_gb300_server* srv,
	unsigned long long id, double* latency_ms, double* queue_ms)
{
	if (!srv) return CVTX_GB300_ST_UNKNOWN;
	return srv->impl.info(id, latency_ms, queue_ms);
}

CVTX_EXPORT int cvtx_gb300_server_stats_get(cvtx_gb300_server* srv,
	cvtx_gb300_server_stats* out)
{
	if (!srv || !out) return -1;
	srv->impl.stats(out);
	return 0;
}

CVTX_EXPORT void cvtx_gb300_server_reset_stats(cvtx_gb300_server* srv) {
	if (srv) srv->impl.reset_stats();
}

CVTX_EXPORT void cvtx_gb300_server_inject_alloc_failures(cvtx_gb300_server* srv, int count) {
	if (srv) srv->impl.inject(count);
}

CVTX_EXPORT void cvtx_gb300_server_destroy(cvtx_gb300_server* srv) {
	delete srv;
}

}  // extern "C"
