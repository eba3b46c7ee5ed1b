#ifndef CVTX_GB300_H
#define CVTX_GB300_H
/*
 * cvtx_gb300.h -- extensions of the GB300 build of cvortex.
 *
 * Nothing here exists in the reference ABI (include/cvortex/libcvtx.h); the
 * reference's ABI functions are unchanged and declared in libcvtx.h. These
 * entry points add what a GPU-resident caller needs:
 *   - an error query (the reference functions return void and fall back to
 *     the CPU silently on OpenCL errors, src/P3D.cpp:352-364; this library
 *     never falls back, it reports instead and writes NaN results);
 *   - a fused vel + dvort call over one particle set;
 *   - a device-pointer API that works on packed records already in GPU
 *     memory, on a caller-supplied CUDA stream (records: see below),
 *     including a device-resident time step;
 *   - many problems in one graph-captured launch (cvtx_gb300_batch_*);
 *   - a serving loop for concurrent clients (cvtx_gb300_server_*);
 *   - the launch-configuration table, FP32 peak probes and a self test of
 *     the device-side failure path.
 *
 * Device record layouts (16-byte aligned arrays of float4):
 *   P3D  : 2 float4 per particle  (x, y, z, volume), (wx, wy, wz, 0)
 *   P2D  : 1 float4 per particle  (x, y, vorticity, area)
 *   F3D  : 2 float4 per filament  (sx, sy, sz, strength), (ex, ey, ez, 0)
 *   point: 1 float4 per point     (x, y, z, 0) or (x, y, 0, 0)
 * Targets are read as tgt[k * tgt_stride] (+1 for the vorticity record), so a
 * P3D source array passed with tgt_stride = 2 serves as its own target set.
 * Outputs are packed float triples / pairs / scalars (the memory layout of
 * bsv_V3f[], bsv_V2f[], float[]).
 *
 * Return codes: 0 success, -1 invalid argument, -2 CUDA error, -3 no GPU
 * enabled, -4 a device-side wait expired (see cvtx_gb300_last_error()).
 */
#include "libcvtx.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Last error message of the GPU path ("" if none) and reset. */
CVTX_EXPORT const char* cvtx_gb300_last_error(void);
CVTX_EXPORT void cvtx_gb300_clear_error(void);

/* Number of CUDA kernels this library has launched since load. */
CVTX_EXPORT unsigned long long cvtx_gb300_kernel_launches(void);

/* Gaussian regularisation: rho below which g(rho)/rho^3 and
 * (3 g/rho^3 - zeta)/rho^2 come from their exact series instead of the
 * reference's erf approximation (which cancels catastrophically there). */
CVTX_EXPORT float cvtx_gb300_gaussian_rho_c(void);
CVTX_EXPORT void cvtx_gb300_set_gaussian_rho_c(float rho_c);

/* Measured FP32 FMA throughput (TFLOP/s, best of `repeats` timed launches of
 * pure-FMA kernels filling every SM) of the first enabled accelerator: the
 * roofline denominator of the all-pairs kernels, which are FP32-pipe bound.
 * _tflops gives the larger of the scalar-FMA and packed (f32x2) FMA probes;
 * _detail gives both. */
CVTX_EXPORT int cvtx_gb300_probe_fp32_tflops(int repeats, double* tflops);
CVTX_EXPORT int cvtx_gb300_probe_fp32_detail(int repeats, double* scalar_fma,
	double* packed_fma);
/* FMA throughput with `packed` f32x2 and `scalar` FP32 FMA chains per thread
 * issued together ((packed, scalar) from a fixed set; -1 otherwise). */
CVTX_EXPORT int cvtx_gb300_probe_fp32_mix(int packed, int scalar, int repeats,
	double* tflops);

/* Launch configurations of the P3D velocity / stretching kernels (targets
 * per thread, threads per CTA, packed two-wide FP32 arithmetic or scalar) and
 * the table that selects one per (reg, ops, target-count bucket); ops: 1 vel,
 * 2 dvort, 3 both; cfg -1 restores the built-in choice. The last
 * configuration is the few-target form (sources spread over the threads of
 * a CTA, reduced in FP64), which the built-in choice takes up to 256 targets,
 * or 2,048 from 262,144 sources; cvtx_gb300_p3d_current_config reports the
 * choice for fewer sources. The autotuner in cvortex_gb300/autotune.py fills
 * the table. */
CVTX_EXPORT int cvtx_gb300_p3d_num_configs(void);
CVTX_EXPORT int cvtx_gb300_p3d_config_info(int cfg, int* tpt, int* nt, int* packed);
CVTX_EXPORT int cvtx_gb300_size_bucket(int n_targets);
CVTX_EXPORT int cvtx_gb300_p3d_set_tuned(int reg, int ops, int bucket, int cfg);
CVTX_EXPORT int cvtx_gb300_p3d_current_config(int reg, int ops, int n_targets);

/* Velocity at and vortex stretching of every particle of one set, in one
 * pass over the pairs: equivalent to cvtx_P3D_M2M_vel(p, n, coords(p), n,
 * vel) followed by cvtx_P3D_M2M_dvort(p, n, p, n, dvort). Either output may
 * be NULL. Returns 0 on success. */
CVTX_EXPORT int cvtx_gb300_P3D_M2M_vel_dvort(const cvtx_P3D** array_start,
	int num_particles, bsv_V3f* vel_out, bsv_V3f* dvort_out,
	const cvtx_VortFunc* kernel, float regularisation_radius);

/* Device-pointer API. `stream` is a cudaStream_t (NULL = legacy default).
 * reg: 0 singular, 1 winckelmans, 2 planetary, 3 gaussian. */
CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M(const void* src, int n_src,
	const void* tgt, int tgt_stride, int n_tgt, float* vel_out,
	float* dvort_out, int reg, float regularisation_radius, void* stream);
/* Workspace in bytes that cvtx_gb300_dev_P3D_M2M allocates (grow-only, per
 * context) for n_tgt targets against n_src particles: self != 0 when the
 * targets are the particles themselves (tgt == src, stride 2); ops 1 vel,
 * 2 dvort, 3 both; form 0 the ordered-pair kernels, form 1 the form the call
 * takes (the self-interaction form where it applies). -1 without an enabled
 * GPU or on bad arguments. */
CVTX_EXPORT long long cvtx_gb300_dev_P3D_M2M_ws_bytes(int n_src, int n_tgt, int self,
	int reg, int ops, int form);
CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_visc(const void* src, int n_src,
	const void* tgt, int tgt_stride, int n_tgt, float* out, int reg,
	float regularisation_radius, float kinematic_visc, void* stream);
/* Vorticity field at points (tgt: records with tgt_stride float4 per point;
 * the first float4 holds the position), with the reference CPU path's
 * 5 sigma box cut-off. Zeros for singular (zeta = 0). */
CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_vort(const void* src, int n_src,
	const void* tgt, int tgt_stride, int n_tgt, float* out, int reg,
	float regularisation_radius, void* stream);
CVTX_EXPORT int cvtx_gb300_dev_P2D_M2M_vel(const void* src, int n_src,
	const void* tgt, int n_tgt, float* out, int reg,
	float regularisation_radius, void* stream);
/* Filament influence matrix: out[i * n_fil + j] = vel_j(mes_i) . dir_i
 * (mes, dir: point records). */
CVTX_EXPORT int cvtx_gb300_dev_F3D_inf_mtrx(const void* fil, int n_fil,
	const void* mes, const void* dir, int n_mes, float* out, void* stream);
/* P2D viscous exchange (zeros for singular / planetary, which have no eta). */
CVTX_EXPORT int cvtx_gb300_dev_P2D_M2M_visc(const void* src, int n_src,
	const void* tgt, int n_tgt, float* out, int reg,
	float regularisation_radius, float kinematic_visc, void* stream);
CVTX_EXPORT int cvtx_gb300_dev_F3D_M2M_vel(const void* fil, int n_fil,
	const void* tgt, int tgt_stride, int n_tgt, float* out, void* stream);
/* Stretching of P3D particles (records, tgt_stride >= 2) by filaments. */
CVTX_EXPORT int cvtx_gb300_dev_F3D_M2M_dvort(const void* fil, int n_fil,
	const void* tgt, int tgt_stride, int n_tgt, float* out, void* stream);
/* cvtx_gb300_dev_P3D_M2M without any device allocation. It has no
 * counterpart in the reference. For callers that cannot let a library call
 * cudaMalloc: device memory owned by one pool reserved up front, or loops
 * that cannot take the latency and synchronisation of cudaMalloc/cudaFree.
 * Split partial sums live in a fixed 32 MiB scratch area inside the library
 * image (held in every GPU's memory while the library is loaded); at most
 * 233,016 targets per call (more: returns -1 with a message), any number of
 * sources. Calls that overlap on the GPU share that scratch and race. The
 * first call on a device resolves the scratch address and should precede any
 * stream capture. The resolved address is kept for the life of the process:
 * do not call this entry point again on a device after cudaDeviceReset on
 * it (the old address may by then belong to another allocation). A
 * device-side wait expiry turns the outputs into NaN. */
CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_noalloc(const void* src, int n_src,
	const void* tgt, int tgt_stride, int n_tgt, float* vel_out,
	float* dvort_out, int reg, float regularisation_radius, void* stream);
/* ---- batched form: many independent P3D problems in one launch ----------
 * Each problem is a device-pointer problem as for cvtx_gb300_dev_P3D_M2M
 * (records as above; dvort needs tgt_stride >= 2). All problems of a batch
 * share the regularisation and ops (1 vel, 2 dvort, 3 both); sigma is per
 * problem. The batch is cut into (problem, target block, source chunk)
 * work items that persistent CTAs claim largest-first, so uneven sizes share
 * the GPU in one launch; results are deterministic. cvtx_gb300_batch_tune
 * times every launch shape x source chunk on the batch and keeps the
 * fastest; cvtx_gb300_batch_capture records the run as a CUDA graph that
 * cvtx_gb300_batch_run then replays. Inputs and outputs must stay valid
 * while the batch exists. */
typedef struct {
	const void* src; int n_src;
	const void* tgt; int tgt_stride; int n_tgt;
	float* vel_out; float* dvort_out;
	float sigma;
} cvtx_gb300_p3d_problem;
typedef struct cvtx_gb300_batch cvtx_gb300_batch;
CVTX_EXPORT cvtx_gb300_batch* cvtx_gb300_batch_create(
	const cvtx_gb300_p3d_problem* problems, int n_problems, int reg, int ops);
CVTX_EXPORT int cvtx_gb300_batch_tune(cvtx_gb300_batch* batch, int repeats);
CVTX_EXPORT int cvtx_gb300_batch_capture(cvtx_gb300_batch* batch);
CVTX_EXPORT int cvtx_gb300_batch_run(cvtx_gb300_batch* batch, void* stream);
CVTX_EXPORT int cvtx_gb300_batch_status(cvtx_gb300_batch* batch);
CVTX_EXPORT int cvtx_gb300_batch_info(const cvtx_gb300_batch* batch, int* tpt,
	int* nt, int* chunk, int* n_items, int* graph, double* interactions);
CVTX_EXPORT void cvtx_gb300_batch_destroy(cvtx_gb300_batch* batch);

/* ---- device-resident time step -------------------------------------------
 * One forward-Euler step of a P3D particle set held on the device as records
 * (stride 2): computes the induced velocity and vorticity rate of every
 * particle (as cvtx_P3D_M2M_vel + cvtx_P3D_M2M_dvort with the set as both
 * sources and targets), then x += dt u, alpha += dt dalpha in place. vel and
 * dvort (3 * n floats each, device) receive the rates at the start of the
 * step. No counterpart in the reference, whose callers integrate on the host. */
CVTX_EXPORT int cvtx_gb300_dev_P3D_step(void* rec, int n, float* vel, float* dvort,
	int reg, float regularisation_radius, float dt, void* stream);

/* ---- serving loop: continuous batching of M2M requests ------------------
 * Requests arrive from any thread (cvtx_gb300_server_submit). A scheduler
 * thread admits them in arrival order as slots and device memory free up:
 * each admitted request takes one slot (CUDA streams at every priority level
 * and a fixed workspace) and a range of one device arena sized by the HBM
 * budget, and runs at a stream priority set by its work per step (smaller
 * runs first on the GPU; set CUDA_DEVICE_MAX_CONNECTIONS=32 before CUDA
 * starts so that the many streams do not share few hardware queues); a
 * request that could never fit the budget is rejected. Its state is copied in
 * once, stays resident for all n_steps time steps (M2M + Euler update on the
 * device), and is copied out once; requests on different slots overlap on the
 * GPU. Results depend only on the request (fixed partition and reduction
 * order), never on what else is in flight. Kinds:
 *   CVTX_GB300_REQ_P3D: state = n P3D records (8 floats: x,y,z,vol, a_x,a_y,a_z,0);
 *       each step vel + dvort of the set on itself, x += dt u, a += dt da.
 *   CVTX_GB300_REQ_P2D: state = n P2D records (4 floats: x,y,Gamma,area);
 *       each step vel of the set on itself, x += dt u.
 *   CVTX_GB300_REQ_F3D: state = n filaments (8 floats: start, strength, end, 0)
 *       fixed, and n_tgt tracer points (4 floats: x,y,z,0) advected by the
 *       filaments' velocity.
 * state_out (same layout as state_in, or the tracer points for F3D) and
 * vel_out (velocity of the last step: 3 or 2 floats per particle / point, or
 * NULL) are written when the request completes. Host buffers may be pageable
 * (staged through pinned memory) or pinned; they must stay valid until the
 * request completes. */
enum {
	CVTX_GB300_REQ_P3D = 0, CVTX_GB300_REQ_P2D = 1, CVTX_GB300_REQ_F3D = 2
};
/* request status */
enum {
	CVTX_GB300_ST_DONE = 0, CVTX_GB300_ST_PENDING = 1, CVTX_GB300_ST_RUNNING = 2,
	CVTX_GB300_ST_REJECTED = -1,      /* larger than the whole HBM budget, or invalid */
	CVTX_GB300_ST_OOM = -2,           /* device memory could not be had */
	CVTX_GB300_ST_FAILED = -3,        /* a CUDA call failed */
	CVTX_GB300_ST_TIMEOUT = -4,       /* a device-side wait expired */
	CVTX_GB300_ST_UNKNOWN = -5        /* no such request */
};
typedef struct {
	int kind;          /* CVTX_GB300_REQ_* */
	int reg;           /* 0 singular, 1 winckelmans, 2 planetary, 3 gaussian */
	float sigma;       /* regularisation radius */
	float dt;          /* time step */
	int n_steps;
	int n;             /* particles, or filaments for F3D */
	int n_tgt;         /* F3D tracer points (ignored otherwise) */
	const float* state_in;
	const float* tgt_in;   /* F3D tracer points */
	float* state_out;
	float* vel_out;
} cvtx_gb300_request;
typedef struct {
	unsigned long long submitted, completed, rejected, failed, queued, in_flight;
	double p50_ms, p99_ms, mean_ms, max_ms;     /* submit -> results in host memory */
	double queue_p50_ms, queue_p99_ms;          /* submit -> admission */
	double interactions;       /* source x target pairs of completed requests */
	double span_s;             /* first submit -> last completion */
	unsigned long long hbm_budget, hbm_used, hbm_peak;
	unsigned long long kernel_launches;
} cvtx_gb300_server_stats;
typedef struct cvtx_gb300_server cvtx_gb300_server;
/* n_slots: concurrent requests (0 = 32, one per hardware work queue at
 * CUDA_DEVICE_MAX_CONNECTIONS=32; each slot holds a 512 MiB split
 * workspace). hbm_bytes: arena size (0 = half of the free device memory, at
 * most 64 GiB). flags: CVTX_GB300_SERVER_DRY_RUN
 * runs the scheduler without a GPU (requests complete at admission without
 * computing; for testing admission logic). */
enum { CVTX_GB300_SERVER_DRY_RUN = 1 };
CVTX_EXPORT cvtx_gb300_server* cvtx_gb300_server_create(int n_slots,
	unsigned long long hbm_bytes, int flags);
/* Returns a request id (> 0), or 0 if the request is invalid. */
CVTX_EXPORT unsigned long long cvtx_gb300_server_submit(cvtx_gb300_server* srv,
	const cvtx_gb300_request* req);
/* Submit reqs[i] at arrival_s[i] seconds after the call (non-decreasing),
 * from the calling thread; ids_out[i] receives the ids. Returns once every
 * request is submitted (not completed). */
CVTX_EXPORT int cvtx_gb300_server_replay(cvtx_gb300_server* srv,
	const cvtx_gb300_request* reqs, const double* arrival_s, int n,
	unsigned long long* ids_out);
/* Wait up to timeout_ms (< 0: no limit) for one request; returns its status. */
CVTX_EXPORT int cvtx_gb300_server_wait(cvtx_gb300_server* srv,
	unsigned long long id, double timeout_ms);
/* Wait for every submitted request; returns 0, or 1 on timeout. */
CVTX_EXPORT int cvtx_gb300_server_drain(cvtx_gb300_server* srv, double timeout_ms);
/* Latency (submit -> done) and queueing delay of a finished request. */
CVTX_EXPORT int cvtx_gb300_server_request_info(cvtx_gb300_server* srv,
	unsigned long long id, double* latency_ms, double* queue_ms);
CVTX_EXPORT int cvtx_gb300_server_stats_get(cvtx_gb300_server* srv,
	cvtx_gb300_server_stats* out);
/* Restart the statistics and forget finished requests (their ids become
 * unknown). Without it a finished request stays queryable until 1,048,576
 * newer ones have finished. */
CVTX_EXPORT void cvtx_gb300_server_reset_stats(cvtx_gb300_server* srv);
/* Host-side fault injection: the next `count` arena allocations fail as if
 * the device were out of memory. */
CVTX_EXPORT void cvtx_gb300_server_inject_alloc_failures(cvtx_gb300_server* srv,
	int count);
/* Drains, then frees every resource. */
CVTX_EXPORT void cvtx_gb300_server_destroy(cvtx_gb300_server* srv);

/* Failure-path self test: one CTA waits, for at most limit_ms (0 < limit_ms
 * <= 1000), on an mbarrier that nothing completes, then records the expiry
 * in an error word the way the all-pairs kernels do. Returns that word
 * (1 = wait expired, the expected answer) or a negative code. */
CVTX_EXPORT int cvtx_gb300_selftest_withheld_wait(double limit_ms);

/* Synchronise `stream`, then read and reset the device error word. Returns 0
 * if no device-side wait expired since the previous check. */
CVTX_EXPORT int cvtx_gb300_dev_status(void* stream);
/* Repack caller AoS arrays already in device memory into records. */
CVTX_EXPORT int cvtx_gb300_dev_pack_P3D(const cvtx_P3D* aos, int n, void* rec,
	void* stream);
CVTX_EXPORT int cvtx_gb300_dev_pack_V3f(const bsv_V3f* pts, int n, void* rec,
	void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CVTX_GB300_H */
