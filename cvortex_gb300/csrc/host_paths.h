// host_paths.h -- host M2M loops (accelerators disabled by the caller, or a
// regularisation bundle with no GPU kernel). See abi_host.cpp.
#pragma once
#include "cvortex/libcvtx.h"

namespace cvtx {
void host_P3D_M2M_vel(const cvtx_P3D** src, int n, const bsv_V3f* mes, int m, bsv_V3f* out,
	const cvtx_VortFunc* k, float sigma);
void host_P3D_M2M_dvort(const cvtx_P3D** src, int n, const cvtx_P3D** ind, int m,
	bsv_V3f* out, const cvtx_VortFunc* k, float sigma);
void host_P3D_M2M_visc_dvort(const cvtx_P3D** src, int n, const cvtx_P3D** ind, int m,
	bsv_V3f* out, const cvtx_VortFunc* k, float sigma, float nu);
void host_P3D_M2M_vort(const cvtx_P3D** src, int n, const bsv_V3f* mes, int m, bsv_V3f* out,
	const cvtx_VortFunc* k, float sigma);
void host_P2D_M2M_vel(const cvtx_P2D** src, int n, const bsv_V2f* mes, int m, bsv_V2f* out,
	const cvtx_VortFunc* k, float sigma);
void host_P2D_M2M_visc_dvort(const cvtx_P2D** src, int n, const cvtx_P2D** ind, int m,
	float* out, const cvtx_VortFunc* k, float sigma, float nu);
void host_F3D_M2M_vel(const cvtx_F3D** fil, int n, const bsv_V3f* mes, int m, bsv_V3f* out);
void host_F3D_M2M_dvort(const cvtx_F3D** fil, int n, const cvtx_P3D** ind, int m, bsv_V3f* out);
void host_F3D_inf_mtrx(const cvtx_F3D** fil, int n, const bsv_V3f* mes, const bsv_V3f* dir,
	int m, float* out);
}  // namespace cvtx
