// tune_api.cpp -- C entry points over the launch-configuration table of the
// P3D induce kernels (p3d.cu). The autotuner (cvortex_gb300/autotune.py)
// times every configuration on representative problems and stores the
// fastest per (regularisation, ops, target-count bucket) with
// cvtx_gb300_p3d_set_tuned.
#include "cvortex/cvtx_gb300.h"
#include "nbody.h"

extern "C" {

CVTX_EXPORT int cvtx_gb300_p3d_num_configs(void) { return cvtx::p3d_induce_num_configs(); }

CVTX_EXPORT int cvtx_gb300_p3d_config_info(int cfg, int* tpt, int* nt, int* packed) {
	if (!tpt || !nt || !packed) return -1;
	return cvtx::p3d_induce_config(cfg, tpt, nt, packed) ? 0 : -1;
}

CVTX_EXPORT int cvtx_gb300_size_bucket(int n_targets) { return cvtx::size_bucket(n_targets); }

CVTX_EXPORT int cvtx_gb300_p3d_set_tuned(int reg, int ops, int bucket, int cfg) {
	return cvtx::p3d_induce_set_tuned(reg, unsigned(ops), bucket, cfg) ? 0 : -1;
}

CVTX_EXPORT int cvtx_gb300_p3d_current_config(int reg, int ops, int n_targets) {
	if (reg < 0 || reg > 3 || ops < 1 || ops > 3) return -1;
	return cvtx::p3d_induce_current_config(reg, unsigned(ops), n_targets);
}

}  // extern "C"
