// p3d_sym_batch.h -- the self-interaction form over many P3D problems at once
// (kernels in p3d_sym.cu, plan and graph in batch.cu): a persistent launch
// over the block-pair items of every problem whose targets are its own
// particles, then one finalize launch over all of their particles.
#pragma once
#include <cstddef>

#include "nbody.h"
#include "p3d_induce.cuh"

namespace cvtx {

// One problem as the kernels read it: blocks of S particles (a multiple of
// 512), nb blocks, slots [nb][NC][n] FP32 (zeroed before every run).
struct alignas(16) SymBatchProblem {
	P3DInduceProblem p;
	InduceConsts kc;
	float* slots;
	int S, nb;
};

// Resident CTAs of the item kernel for (reg, ops) on one SM.
int p3d_sym_batch_occupancy(int reg, unsigned ops);

// Items are int4 (problem, bi, bj, 0), bi <= bj. prefix[i] is the first
// global particle index of problem i (prefix[n_probs] = total). Enqueues the
// item kernel (grid CTAs, `next` zeroed by the caller) and the finalize
// kernel on `s`.
cudaError_t p3d_sym_batch_enqueue(int reg, unsigned ops, const SymBatchProblem* probs,
	int n_probs, const int4* items, int n_items, const int* prefix, int total, unsigned* next,
	unsigned* err, int grid, cudaStream_t s);

}  // namespace cvtx
