// redist.h -- particle redistribution (remeshing) onto a regular grid.
//
// Restates the reference's cvtx_P3D_redistribute_on_grid /
// cvtx_P2D_redistribute_on_grid (src/P3D.cpp:508-634, src/P2D.cpp:283-404):
//   1. grid: corner `min` (bounding-box minimum moved out by the stencil
//      radius, then snapped so that the particle mean lies 5 + round(.) cells
//      from it), spacing gd = grid_density;
//   2. every particle spreads alpha * f(U) f(W) f(V) onto the (2R+1)^d grid
//      points around its nearest point (R = round(redistributor radius);
//      U, W, V the axis distances in cells); exactly zero contributions are
//      dropped;
//   3. contributions to the same grid point are summed; the new particles
//      come out in ascending Morton order of their grid keys (bit b of x, y,
//      z at bits 3b, 3b+1, 3b+2) -- the depth-first order of the reference's
//      octree / quadtree;
//   4. particles with strength <= mean strength * negligible_vort are removed
//      and their vorticity is spread evenly over the survivors; if more than
//      max_output_particles remain, a strength threshold found by the
//      reference's histogram search removes more in the same way.
// Sums run in FP64 in particle order (the reference sums in FP32 per OpenMP
// thread, so its last bits depend on the thread count). Host and GPU paths
// produce the same cells bit for bit.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "cvortex/libcvtx.h"

namespace cvtx {

// Id of a redistribution function made by this library's cvtx_RedistFunc_*
// factories (0 lambda0, 1 lambda1, 2 lambda2, 3 lambda3, 4 m4p), or -1.
int redist_kind(const cvtx_RedistFunc* f);

struct RedistGrid {
	int dims = 3;          // 2 or 3
	float min[3] = {0.f, 0.f, 0.f};
	float gd = 1.f;        // grid spacing
	float rgd = 1.f;       // 1 / gd in FP32, as the reference computes it
	int radius = 0;        // stencil half width in cells
	int bits = 21;         // Morton bits per axis
};

// Grid cells with their summed vorticity (vort: dims == 3 -> 3 per cell,
// dims == 2 -> 1 per cell), ascending Morton code. `code` and `vort` point
// into the vectors below (host path) or into pinned memory that the GPU
// path copied them to.
struct RedistCells {
	const uint64_t* code = nullptr;
	const float* vort = nullptr;
	size_t n = 0;
	std::vector<uint64_t> code_v;
	std::vector<float> vort_v;
};

// Particles as flat arrays: pos (dims per particle), str (3 or 1 per particle).
bool redist_grid(int dims, const float* pos, int n, const cvtx_RedistFunc* f, float gd,
	RedistGrid* g);
void redist_cells_host(const RedistGrid& g, const cvtx_RedistFunc* f, const float* pos,
	const float* str, int n, RedistCells* out);
// GPU path (kind from redist_kind >= 0). Device scratch comes from `scratch`
// and the cells are copied to `pinned` (both grow-only, kept between calls:
// a 200,000-particle M4' call needs ~1.5 GB and 25 MB).
struct DevBuf;
struct HostBuf;
cudaError_t redist_cells_gpu(const RedistGrid& g, int kind, const float* pos, const float* str,
	int n, RedistCells* out, DevBuf* scratch, HostBuf* pinned, cudaStream_t stream);

// Morton helpers shared by both paths.
inline uint64_t spread3(uint32_t v) {
	uint64_t x = v & 0x1fffffu;
	x = (x | (x << 32)) & 0x1f00000000ffffull;
	x = (x | (x << 16)) & 0x1f0000ff0000ffull;
	x = (x | (x << 8)) & 0x100f00f00f00f00full;
	x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
	x = (x | (x << 2)) & 0x1249249249249249ull;
	return x;
}
inline uint32_t gather3(uint64_t x) {
	x &= 0x1249249249249249ull;
	x = (x | (x >> 2)) & 0x10c30c30c30c30c3ull;
	x = (x | (x >> 4)) & 0x100f00f00f00f00full;
	x = (x | (x >> 8)) & 0x1f0000ff0000ffull;
	x = (x | (x >> 16)) & 0x1f00000000ffffull;
	x = (x | (x >> 32)) & 0x1fffffull;
	return uint32_t(x);
}
inline uint64_t spread2(uint32_t v) {
	uint64_t x = v;
	x = (x | (x << 16)) & 0x0000ffff0000ffffull;
	x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
	x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
	x = (x | (x << 2)) & 0x3333333333333333ull;
	x = (x | (x << 1)) & 0x5555555555555555ull;
	return x;
}
inline uint32_t gather2(uint64_t x) {
	x &= 0x5555555555555555ull;
	x = (x | (x >> 1)) & 0x3333333333333333ull;
	x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
	x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
	x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
	x = (x | (x >> 16)) & 0x00000000ffffffffull;
	return uint32_t(x);
}

}  // namespace cvtx
