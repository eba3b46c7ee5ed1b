// nbody.h -- host-side interface of the all-pairs kernels (sm_103a).
//
// Device data layout (packed once per call by the host runtime or by the
// caller of the device-pointer API):
//   P3D record: 2 float4 = (x, y, z, volume), (alpha_x, alpha_y, alpha_z, 0)
//   P2D record: 1 float4 = (x, y, Gamma, area)
//   F3D record: 2 float4 = (start_x, start_y, start_z, strength),
//                          (end_x, end_y, end_z, 0)
//   Measurement points:    float4 (x, y, z, 0) or (x, y, 0, 0)
// Targets are addressed as tgt[k * tstride] (position record) and
// tgt[k * tstride + 1] (vorticity record), so a source array with stride 2
// can serve directly as the target array when the caller aliases them.
// Outputs are written as packed float3 / float2 / float arrays, which is the
// memory layout of bsv_V3f[] / bsv_V2f[] / float[] on the host.
//
// Every launcher takes a caller-provided workspace (for split-source partial
// sums) whose required size is returned by the matching *_ws_bytes query for
// the same arguments; the launchers never allocate.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace cvtx {

enum : unsigned { kOpVel = 1u, kOpDvort = 2u };

struct P3DInduceProblem {
	const float4* src; int n_src;
	const float4* tgt; int tstride; int n_tgt;
	float* out_vel;     // 3 * n_tgt floats, or nullptr
	float* out_dvort;   // 3 * n_tgt floats, or nullptr (needs target vorticity)
	float sigma;
};

struct P3DViscProblem {
	const float4* src; int n_src;
	const float4* tgt; int tstride; int n_tgt;
	float* out;         // 3 * n_tgt floats
	float sigma, nu;
};

struct P3DVortProblem {
	const float4* src; int n_src;
	const float4* tgt; int tstride; int n_tgt;
	float* out;         // 3 * n_tgt floats
	float sigma;
};

struct P2DVelProblem {
	const float4* src; int n_src;
	const float4* tgt; int n_tgt;   // tgt: (x, y, *, *)
	float* out;         // 2 * n_tgt floats
	float sigma;
};

struct P2DViscProblem {
	const float4* src; int n_src;
	const float4* tgt; int n_tgt;   // tgt: (x, y, Gamma, area)
	float* out;         // n_tgt floats
	float sigma, nu;
};

struct F3DVelProblem {
	const float4* fil; int n_fil;
	const float4* tgt; int tstride; int n_tgt;
	float* out;         // 3 * n_tgt floats
};

struct F3DDvortProblem {
	const float4* fil; int n_fil;
	const float4* tgt; int tstride; int n_tgt;   // P3D records
	float* out;         // 3 * n_tgt floats
};

struct F3DInfProblem {
	const float4* fil; int n_fil;
	const float4* mes; int n_mes;   // (x, y, z, 0)
	const float4* dir;              // (x, y, z, 0)
	float* out;                     // n_mes * n_fil floats, row-major by mes
};

struct LaunchEnv {
	void* ws;            // workspace, 256-byte aligned
	size_t ws_bytes;
	unsigned* err;       // device error word (0 = ok)
	cudaStream_t stream;
	int num_sms;
	// When set, launchers cap the number of source splits so that the split
	// partials fit ws_bytes (for callers with a fixed-size workspace).
	bool cap_to_ws = false;
	// When > 0, the P3D / P2D / F3D velocity launchers use at least
	// ceil(n_src / cta_src_cap) source splits (within the caps above), which
	// bounds how long one CTA holds its SM: the CUDA block scheduler does not
	// preempt running CTAs, so this bounds how long a higher-priority launch
	// waits for one.
	int cta_src_cap = 0;
};

// The fewest source splits a launch takes under env.cta_src_cap.
inline int min_split_for(const LaunchEnv& env, int n_src) {
	return env.cta_src_cap > 0 ? (n_src + env.cta_src_cap - 1) / env.cta_src_cap : 1;
}

// Largest split count whose FP64 partials (nc sums per target) fit `ws_bytes`.
inline int split_cap_for(size_t ws_bytes, int nc, int n_tgt) {
	const size_t per = size_t(nc) * size_t(n_tgt > 0 ? n_tgt : 1) * sizeof(double);
	const size_t cap = ws_bytes / per;
	return cap < 1 ? 1 : (cap > 64 ? 64 : int(cap));
}

// Kernel-launch counter shared by every launcher (for the launch statistics
// exposed by the library).
void count_launch(int n = 1);
unsigned long long launch_count();

// Regularisation id from the reference tag string; -1 if not GPU-capable.
// Tags: "singular" 0, "winckelmans" 1, "planetary" 2, "gaussian" 3.
int reg_from_tag(const char* tag);

// Gaussian small-rho threshold (rho below which the series is used).
float gaussian_rho_c();
void set_gaussian_rho_c(float rho_c);

size_t p3d_induce_ws_bytes(int reg, unsigned ops, int n_src, int n_tgt, int num_sms);
// Workspace for p3d_induce on this problem: as above, or the larger
// workspace of the self-interaction form when that form applies to it.
size_t p3d_induce_ws_bytes_for(int reg, unsigned ops, const P3DInduceProblem& p, int num_sms);
cudaError_t p3d_induce(int reg, unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env);

// Self-interaction form (p3d_sym.cu): the particles are their own targets
// (tgt == src, stride 2, n_tgt == n_src, at least CVTX_GB300_SYM_MIN
// particles, default 16,384), so each unordered pair is evaluated once.
// p3d_induce takes it when it applies, the launch is not bound by a CTA
// lifetime cap (env.cta_src_cap), no launch configuration is forced, and the
// workspace suffices; results stay deterministic. p3d_self_ws_bytes is
// SIZE_MAX where the workspace cap would leave too few work items for the
// GPU (the ordered-pair kernels then serve the call).
bool p3d_self_form_applies(int reg, unsigned ops, const P3DInduceProblem& p);
size_t p3d_self_ws_bytes(int reg, unsigned ops, int n, int num_sms, size_t ws_cap = 0);
cudaError_t p3d_self(int reg, unsigned ops, const P3DInduceProblem& p, const LaunchEnv& env);

// As p3d_induce, with the source-split count capped so that the partial sums
// fit env.ws_bytes (a fixed scratch area); never needs more than that.
cudaError_t p3d_induce_bounded(int reg, unsigned ops, const P3DInduceProblem& p,
	const LaunchEnv& env);

// Launch configurations of the induce kernels (targets per thread, threads
// per CTA, packed f32x2 arithmetic) and the tuning table that selects one per
// (regularisation, ops, target-count bucket).
constexpr int kNumSizeBuckets = 6;
inline int size_bucket(int n_tgt) {
	return n_tgt < 8192 ? 0 : n_tgt < 32768 ? 1 : n_tgt < 131072 ? 2 : n_tgt < 524288 ? 3
		: n_tgt < 2097152 ? 4 : 5;
}
int p3d_induce_num_configs();
bool p3d_induce_config(int cfg, int* tpt, int* nt, int* packed);
bool p3d_induce_set_tuned(int reg, unsigned ops, int bucket, int cfg);
int p3d_induce_current_config(int reg, unsigned ops, int n_tgt);

size_t p3d_visc_ws_bytes(int reg, int n_src, int n_tgt, int num_sms);
// Workspace for p3d_visc on this problem (the self-interaction form's when
// it applies).
size_t p3d_visc_ws_bytes_for(int reg, const P3DViscProblem& p, int num_sms);
cudaError_t p3d_visc(int reg, const P3DViscProblem& p, const LaunchEnv& env);
// Self-interaction form of the viscous exchange (p3d_sym.cu), on the same
// conditions as p3d_self_form_applies; p3d_visc takes it when it applies and
// the workspace suffices.
bool p3d_visc_self_form_applies(int reg, const P3DViscProblem& p);
size_t p3d_visc_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap = 0);
cudaError_t p3d_visc_self(int reg, const P3DViscProblem& p, const LaunchEnv& env);

size_t p3d_vort_ws_bytes(int reg, int n_src, int n_tgt, int num_sms);
size_t p3d_vort_ws_bytes_for(int reg, const P3DVortProblem& p, int num_sms);
cudaError_t p3d_vort(int reg, const P3DVortProblem& p, const LaunchEnv& env);
// The vorticity field at the particles' own positions (p3d_sym.cu), under
// the conditions of p3d_self_form_applies (Winckelmans, planetary,
// Gaussian; no configuration forced by CVTX_GB300_VORT_CFG).
bool p3d_vort_self_form_applies(int reg, const P3DVortProblem& p);
size_t p3d_vort_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap = 0);
cudaError_t p3d_vort_self(int reg, const P3DVortProblem& p, const LaunchEnv& env);

size_t p2d_vel_ws_bytes(int reg, int n_src, int n_tgt, int num_sms);
// As above, or the larger workspace of the self-interaction form when that
// form applies to the problem (the same rule for the viscous exchange).
size_t p2d_vel_ws_bytes_for(int reg, const P2DVelProblem& p, int num_sms);
cudaError_t p2d_vel(int reg, const P2DVelProblem& p, const LaunchEnv& env);
// The velocity scale of the reference (1/(2 pi), with 1/sigma^2 for the
// rho-normalised regularisations).
double p2d_vel_scale(int reg, float sigma);

size_t p2d_visc_ws_bytes(int reg, int n_src, int n_tgt, int num_sms);
size_t p2d_visc_ws_bytes_for(int reg, const P2DViscProblem& p, int num_sms);
cudaError_t p2d_visc(int reg, const P2DViscProblem& p, const LaunchEnv& env);

// P2D self-interaction form (p2d_sym.cu): the records are their own targets
// (tgt == src, n_tgt == n_src, at least CVTX_GB300_SYM_MIN particles), each
// unordered pair evaluated once. p2d_vel / p2d_visc take it under the same
// conditions as p3d_induce takes the P3D form (and, for the velocity, no
// launch configuration forced by CVTX_GB300_P2D_CFG); *_self_ws_bytes is
// SIZE_MAX where the workspace cap would leave too few work items.
bool p2d_vel_self_form_applies(const P2DVelProblem& p);
size_t p2d_vel_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap = 0);
cudaError_t p2d_vel_self(int reg, const P2DVelProblem& p, const LaunchEnv& env);
bool p2d_visc_self_form_applies(int reg, const P2DViscProblem& p);
size_t p2d_visc_self_ws_bytes(int reg, int n, int num_sms, size_t ws_cap = 0);
cudaError_t p2d_visc_self(int reg, const P2DViscProblem& p, const LaunchEnv& env);

size_t f3d_vel_ws_bytes(int n_fil, int n_tgt, int num_sms);
cudaError_t f3d_vel(const F3DVelProblem& p, const LaunchEnv& env);

size_t f3d_dvort_ws_bytes(int n_fil, int n_tgt, int num_sms);
cudaError_t f3d_dvort(const F3DDvortProblem& p, const LaunchEnv& env);

cudaError_t f3d_inf_mtrx(const F3DInfProblem& p, const LaunchEnv& env);

// Repack kernels: caller AoS records (already on the device) -> records above.
cudaError_t pack_p3d(const void* aos28, int n, float4* out, cudaStream_t s);
cudaError_t pack_p2d(const void* aos16, int n, float4* out, cudaStream_t s);
cudaError_t pack_f3d(const void* aos28, int n, float4* out, cudaStream_t s);
cudaError_t pack_v3(const void* v12, int n, float4* out, cudaStream_t s);
cudaError_t pack_v2(const void* v8, int n, float4* out, cudaStream_t s);
// Gather through a device-visible array of record pointers.
cudaError_t gather_p3d(const void* const* ptrs, int n, float4* out, cudaStream_t s);

// Forward-Euler update of resident state (advance.cu): positions move by
// dt * vel (packed float3 / float2); P3D vorticity moves by dt * dvort when
// dvort is non-null.
cudaError_t advance_p3d(float4* rec, int n, const float* vel, const float* dvort, float dt,
	cudaStream_t s);
cudaError_t advance_p2d(float4* rec, int n, const float* vel, float dt, cudaStream_t s);
cudaError_t advance_points(float4* pts, int n, const float* vel, float dt, cudaStream_t s);

}  // namespace cvtx
