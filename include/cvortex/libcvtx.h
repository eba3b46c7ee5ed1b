#ifndef CVTX_LIBCVTX_H
#define CVTX_LIBCVTX_H
/*
 * libcvtx.h -- the cvtx_ C ABI served by the GB300 build of cvortex.
 *
 * Every type and function declared here keeps the layout, name, argument
 * order and meaning of the reference header (cvortex 0.3.8,
 * include/cvortex/libcvtx.h), so that existing callers (C, Julia ccall,
 * Python ctypes) link against libcvortex.so unchanged. Line numbers after
 * each group cite that reference header.
 *
 * The declarations follow the cvortex header, Copyright (c) 2019 HJA Bird,
 * distributed under the MIT licence.
 *
 * Hot path served by CUDA kernels for sm_103a when an accelerator is enabled:
 *   cvtx_P3D_M2M_vel / _dvort / _visc_dvort / _vort
 *   cvtx_P2D_M2M_vel / _visc_dvort
 *   cvtx_F3D_M2M_vel / _dvort, cvtx_F3D_inf_mtrx
 * All other entry points are host code. GB300-specific extensions (error
 * query, device-pointer API, batched and serving forms) are declared in
 * cvtx_gb300.h, not here.
 */

#ifndef CVTX_EXPORT
# ifdef _WIN32
#  define CVTX_EXPORT __declspec(dllimport)
# else
#  define CVTX_EXPORT
# endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

#include <bsv/bsv.h>

/* Types (reference libcvtx.h:52-99). Sizes: cvtx_P3D 28 B, cvtx_F3D 28 B,
 * cvtx_P2D 16 B; no padding. */
typedef struct {
	bsv_V3f coord;
	bsv_V3f vorticity;
	float volume;
} cvtx_P3D;

typedef struct {
	bsv_V3f start, end;   /* segment end points */
	float strength;       /* vorticity per unit length */
} cvtx_F3D;

typedef struct {
	bsv_V2f coord;
	float vorticity;
	float area;
} cvtx_P2D;

/* Regularisation bundle (reference libcvtx.h:86-94). The host paths call the
 * function pointers; the GPU path dispatches on cl_kernel_name_ext
 * ("singular", "winckelmans", "planetary", "gaussian"). Any other tag, e.g.
 * a caller-built bundle with "" as the tag, runs on the host through the
 * caller's function pointers, as in the reference. */
typedef struct {
	float (*g_3D)(float rho);
	float (*g_2D)(float rho);
	float (*zeta_3D)(float rho);
	void (*combined_3D)(float rho, float* g, float* zeta);
	float (*eta_3D)(float rho);
	float (*eta_2D)(float rho);
	char cl_kernel_name_ext[32];
} cvtx_VortFunc;

typedef struct {
	float (*func)(float U);
	float radius;
} cvtx_RedistFunc;

/* Library and accelerator control (reference libcvtx.h:101-110). */
CVTX_EXPORT void cvtx_initialise();
CVTX_EXPORT void cvtx_finalise();
CVTX_EXPORT const char* cvtx_information();
CVTX_EXPORT int cvtx_num_accelerators();
CVTX_EXPORT int cvtx_num_enabled_accelerators();
CVTX_EXPORT const char* cvtx_accelerator_name(int accelerator_id);
CVTX_EXPORT int cvtx_accelerator_enabled(int accelerator_id);
CVTX_EXPORT void cvtx_accelerator_enable(int accelerator_id);
CVTX_EXPORT void cvtx_accelerator_disable(int accelerator_id);

/* Regularisation constructors (reference libcvtx.h:112-123). */
CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_singular(void);
CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_winckelmans(void);
CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_planetary(void);
CVTX_EXPORT const cvtx_VortFunc cvtx_VortFunc_gaussian(void);

CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda0(void);
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda1(void);
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda2(void);
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_lambda3(void);
CVTX_EXPORT const cvtx_RedistFunc cvtx_RedistFunc_m4p(void);

/* 3D vortex particles (reference libcvtx.h:125-264). */
CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_vel(const cvtx_P3D* self,
	const bsv_V3f mes_point, const cvtx_VortFunc* kernel,
	float regularisation_radius);
CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_dvort(const cvtx_P3D* self,
	const cvtx_P3D* induced_particle, const cvtx_VortFunc* kernel,
	float regularisation_radius);
CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_visc_dvort(const cvtx_P3D* self,
	const cvtx_P3D* induced_particle, const cvtx_VortFunc* kernel,
	float regularisation_radius, float kinematic_visc);
CVTX_EXPORT bsv_V3f cvtx_P3D_S2S_vort(const cvtx_P3D* self,
	const bsv_V3f mes_point, const cvtx_VortFunc* kernel,
	float regularisation_radius);

CVTX_EXPORT void cvtx_P3D_S2M_vel(const cvtx_P3D* self,
	const bsv_V3f* mes_start, const int num_mes, bsv_V3f* result_array,
	const cvtx_VortFunc* kernel, float regularisation_radius);
CVTX_EXPORT void cvtx_P3D_S2M_dvort(const cvtx_P3D* self,
	const cvtx_P3D** induced_start, const int num_induced,
	bsv_V3f* result_array, const cvtx_VortFunc* kernel,
	float regularisation_radius);
CVTX_EXPORT void cvtx_P3D_S2M_visc_dvort(const cvtx_P3D* self,
	const cvtx_P3D** induced_start, const int num_induced,
	bsv_V3f* result_array, const cvtx_VortFunc* kernel,
	float regularisation_radius, float kinematic_visc);
CVTX_EXPORT void cvtx_P3D_S2M_vort(const cvtx_P3D* self,
	const bsv_V3f* mes_start, const int num_mes, bsv_V3f* result_array,
	const cvtx_VortFunc* kernel, float regularisation_radius);

CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_vel(const cvtx_P3D** array_start,
	const int num_particles, const bsv_V3f mes_point,
	const cvtx_VortFunc* kernel, float regularisation_radius);
CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_dvort(const cvtx_P3D** array_start,
	const int num_particles, const cvtx_P3D* induced_particle,
	const cvtx_VortFunc* kernel, float regularisation_radius);
CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_visc_dvort(const cvtx_P3D** array_start,
	const int num_particles, const cvtx_P3D* induced_particle,
	const cvtx_VortFunc* kernel, float regularisation_radius,
	float kinematic_visc);
CVTX_EXPORT bsv_V3f cvtx_P3D_M2S_vort(const cvtx_P3D** array_start,
	const int num_particles, const bsv_V3f mes_point,
	const cvtx_VortFunc* kernel, float regularisation_radius);

/* M2M: every source against every target. GPU-backed here (the hot path);
 * each replaces the reference declaration and implementation cited. */
/* reference libcvtx.h:213-220; src/P3D.cpp:343-366 (GPU: src/ocl_P3D.cpp:150-321) */
CVTX_EXPORT void cvtx_P3D_M2M_vel(const cvtx_P3D** array_start,
	const int num_particles, const bsv_V3f* mes_start, const int num_mes,
	bsv_V3f* result_array, const cvtx_VortFunc* kernel,
	float regularisation_radius);
/* reference libcvtx.h:222-229; src/P3D.cpp:387-410 (GPU: src/ocl_P3D.cpp:323-506) */
CVTX_EXPORT void cvtx_P3D_M2M_dvort(const cvtx_P3D** array_start,
	const int num_particles, const cvtx_P3D** induced_start,
	const int num_induced, bsv_V3f* result_array,
	const cvtx_VortFunc* kernel, float regularisation_radius);
/* reference libcvtx.h:231-239; src/P3D.cpp:432-456 (GPU: src/ocl_P3D.cpp:508-725) */
CVTX_EXPORT void cvtx_P3D_M2M_visc_dvort(const cvtx_P3D** array_start,
	const int num_particles, const cvtx_P3D** induced_start,
	const int num_induced, bsv_V3f* result_array,
	const cvtx_VortFunc* kernel, float regularisation_radius,
	float kinematic_visc);
/* reference libcvtx.h:241-248; src/P3D.cpp:476-498 (GPU: src/ocl_P3D.cpp:728-899) */
CVTX_EXPORT void cvtx_P3D_M2M_vort(const cvtx_P3D** array_start,
	const int num_particles, const bsv_V3f* mes_start, const int num_mes,
	bsv_V3f* result_array, const cvtx_VortFunc* kernel,
	float regularisation_radius);

/* reference libcvtx.h:250-257; src/P3D.cpp:508-634 */
CVTX_EXPORT int cvtx_P3D_redistribute_on_grid(
	const cvtx_P3D** input_array_start, const int n_input_particles,
	cvtx_P3D* output_particles, int max_output_particles,
	const cvtx_RedistFunc* redistributor, float grid_density,
	float negligible_vort);
/* reference libcvtx.h:259-264; src/P3D.cpp:669-707 */
CVTX_EXPORT void cvtx_P3D_pedrizzetti_relaxation(
	cvtx_P3D** input_array_start, const int n_input_particles, float fdt,
	const cvtx_VortFunc* kernel, float regularisation_radius);

/* Straight singular vortex filaments (reference libcvtx.h:266-305). */
CVTX_EXPORT bsv_V3f cvtx_F3D_S2S_vel(const cvtx_F3D* self,
	const bsv_V3f mes_point);
CVTX_EXPORT bsv_V3f cvtx_F3D_S2S_dvort(const cvtx_F3D* self,
	const cvtx_P3D* induced_particle);
CVTX_EXPORT bsv_V3f cvtx_F3D_M2S_vel(const cvtx_F3D** array_start,
	const int num_filaments, const bsv_V3f mes_point);
CVTX_EXPORT bsv_V3f cvtx_F3D_M2S_dvort(const cvtx_F3D** array_start,
	const int num_filaments, const cvtx_P3D* induced_particle);
/* reference libcvtx.h:285-290; src/F3D.cpp:162-180 (GPU: src/ocl_F3D.cpp:36-420) */
CVTX_EXPORT void cvtx_F3D_M2M_vel(const cvtx_F3D** array_start,
	const int num_filaments, const bsv_V3f* mes_start, const int num_mes,
	bsv_V3f* result_array);
/* reference libcvtx.h:292-297; src/F3D.cpp:182-202 (GPU: src/ocl_F3D.cpp:422-646) */
CVTX_EXPORT void cvtx_F3D_M2M_dvort(const cvtx_F3D** array_start,
	const int num_filaments, const cvtx_P3D** induced_start,
	const int num_induced, bsv_V3f* result_array);
/* reference libcvtx.h:299-305; src/F3D.cpp:204-227 (CPU only there) */
CVTX_EXPORT void cvtx_F3D_inf_mtrx(const cvtx_F3D** array_start,
	const int num_filaments, const bsv_V3f* mes_start,
	const bsv_V3f* dir_start, const int num_mes, float* result_matrix);

/* 2D vortex particles (reference libcvtx.h:307-379). */
CVTX_EXPORT bsv_V2f cvtx_P2D_S2S_vel(const cvtx_P2D* self,
	const bsv_V2f mes_point, const cvtx_VortFunc* kernel,
	float regularisation_radius);
CVTX_EXPORT void cvtx_P2D_S2M_vel(const cvtx_P2D* self,
	const bsv_V2f* mes_start, const int num_mes, bsv_V2f* result_array,
	const cvtx_VortFunc* kernel, float regularisation_radius);
CVTX_EXPORT bsv_V2f cvtx_P2D_M2S_vel(const cvtx_P2D** array_start,
	const int num_particles, const bsv_V2f mes_point,
	const cvtx_VortFunc* kernel, float regularisation_radius);
/* reference libcvtx.h:329-336; src/P2D.cpp:141-162 (GPU: src/ocl_P2D.cpp:37-424) */
CVTX_EXPORT void cvtx_P2D_M2M_vel(const cvtx_P2D** array_start,
	const int num_particles, const bsv_V2f* mes_start, const int num_mes,
	bsv_V2f* result_array, const cvtx_VortFunc* kernel,
	float regularisation_radius);
CVTX_EXPORT float cvtx_P2D_S2S_visc_dvort(const cvtx_P2D* self,
	const cvtx_P2D* induced_particle, const cvtx_VortFunc* kernel,
	float regularisation_radius, float kinematic_visc);
CVTX_EXPORT void cvtx_P2D_S2M_visc_dvort(const cvtx_P2D* self,
	const cvtx_P2D** induced_start, const int num_induced,
	float* result_array, const cvtx_VortFunc* kernel,
	float regularisation_radius, float kinematic_visc);
CVTX_EXPORT float cvtx_P2D_M2S_visc_dvort(const cvtx_P2D** array_start,
	const int num_particles, const cvtx_P2D* induced_particle,
	const cvtx_VortFunc* kernel, float regularisation_radius,
	float kinematic_visc);
/* reference libcvtx.h:362-370; src/P2D.cpp:252-276 (GPU: src/ocl_P2D.cpp:426-631) */
CVTX_EXPORT void cvtx_P2D_M2M_visc_dvort(const cvtx_P2D** array_start,
	const int num_particles, const cvtx_P2D** induced_start,
	const int num_induced, float* result_array,
	const cvtx_VortFunc* kernel, float regularisation_radius,
	float kinematic_visc);
/* reference libcvtx.h:372-379; src/P2D.cpp:283-404 */
CVTX_EXPORT int cvtx_P2D_redistribute_on_grid(
	const cvtx_P2D** input_array_start, const int num_particles,
	cvtx_P2D* output_particles, int num_output_particles,
	const cvtx_RedistFunc* redistributor, float grid_density,
	float negligible_vort);

#ifdef __cplusplus
}
#endif
#endif /* CVTX_LIBCVTX_H */
