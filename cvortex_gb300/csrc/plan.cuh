// plan.cuh -- launch planning shared by the all-pairs launchers.
//
// A problem of n_tgt targets and n_src sources is cut into target blocks
// (TPT * NT targets, one CTA each) and source splits. Splits exist so that
// problems with few target blocks still fill all SMs and so that the total
// CTA count lands close to a whole number of waves (resident CTAs per wave =
// SMs x CTAs per SM from the occupancy calculator). Split partial sums go to
// the workspace as FP64 and are combined in a fixed order by a finalize
// kernel, so results do not depend on scheduling.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cuda_runtime.h>

namespace cvtx {

struct Plan {
	int n_tblocks = 0;     // CTAs along x (target blocks)
	int n_split = 1;       // CTAs along y (source splits)
	int src_per_split = 0; // sources per split (multiple of the tile)
	size_t smem = 0;       // dynamic shared memory per CTA
	size_t ws_bytes = 0;   // FP64 partials: n_split * NC * n_tgt * 8 (0 if one split)
};

// Resident CTAs per SM for `kernel` at `nt` threads and `smem` bytes; sets the
// dynamic shared memory limit of the kernel on first use.
template <class K>
inline int resident_ctas(K kernel, int nt, size_t smem) {
	if (smem > 48 * 1024)
		cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
	int occ = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, nt, smem) != cudaSuccess || occ < 1)
		occ = 1;
	return occ;
}

inline Plan make_plan(int n_src, int n_tgt, int targets_per_cta, int tile, int nc,
	int capacity, size_t smem, int max_split = 64, int min_split = 1)
{
	Plan pl;
	pl.smem = smem;
	pl.n_tblocks = (n_tgt + targets_per_cta - 1) / targets_per_cta;
	if (pl.n_tblocks < 1) pl.n_tblocks = 1;
	// At least four tiles of sources per split keeps the copy pipeline busy.
	int cap_split = n_src / (4 * tile);
	cap_split = std::max(1, std::min(max_split, cap_split));
	// min_split: the caller's bound on sources per CTA, within the caps
	const int lo_split = std::max(1, std::min(min_split, cap_split));
	int best_s = lo_split;
	double best_eff = -1.0;
	for (int s = lo_split; s <= cap_split; ++s) {
		const double waves = double(pl.n_tblocks) * s / double(capacity);
		const double eff = waves / std::ceil(waves);
		if (eff > best_eff + 0.02) { best_eff = eff; best_s = s; }
		if (best_eff >= 0.97) break;
	}
	int per = (n_src + best_s - 1) / best_s;
	per = ((per + tile - 1) / tile) * tile;
	if (per < tile) per = tile;
	pl.src_per_split = per;
	pl.n_split = std::max(1, (n_src + per - 1) / per);
	pl.ws_bytes = pl.n_split > 1 ? size_t(pl.n_split) * nc * size_t(n_tgt) * sizeof(double) : 0;
	return pl;
}

}  // namespace cvtx
