#ifndef CVTX_GB300_H
#define CVTX_GB300_H
/*
 * cvtx_gb300.h -- extensions of the GB300 build of cvortex.
 *
 * Nothing here exists in the reference ABI (include/cvortex/libcvtx.h); the
 * reference's ABI functions are unchanged and declared in libcvtx.h. These
 * entry points add what a GPU-resident caller needs:
 *   - an error query (the reference functions return void and fall back to
 *     the CPU silently on OpenCL errors, src/P3D.cpp:352-364; this build
 *     never falls back, it reports instead and writes NaN results);
 *   - a fused vel + dvort call over one particle set;
 *   - a device-pointer API that works on packed records already in GPU
 *     memory, on a caller-supplied CUDA stream (records: see below).
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
CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_visc(const void* src, int n_src,
	const void* tgt, int tgt_stride, int n_tgt, float* out, int reg,
	float regularisation_radius, float kinematic_visc, void* stream);
CVTX_EXPORT int cvtx_gb300_dev_P2D_M2M_vel(const void* src, int n_src,
	const void* tgt, int n_tgt, float* out, int reg,
	float regularisation_radius, void* stream);
CVTX_EXPORT int cvtx_gb300_dev_F3D_M2M_vel(const void* fil, int n_fil,
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
 * stream capture. A device-side wait expiry turns the outputs into NaN. */
CVTX_EXPORT int cvtx_gb300_dev_P3D_M2M_noalloc(const void* src, int n_src,
	const void* tgt, int tgt_stride, int n_tgt, float* vel_out,
	float* dvort_out, int reg, float regularisation_radius, void* stream);
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
