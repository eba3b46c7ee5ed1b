// redist.cu -- GPU part of particle redistribution (see redist.h).
//
//   spread:   one thread per (particle, stencil point): grid key, Morton code
//             and the contribution alpha f(U) f(W) f(V); an exactly zero
//             contribution gets a code above every real one;
//   sort:     stable radix sort of (code, entry index) over the code bits in
//             use (CUB), so that a grid point's entries stay in particle order;
//   sum:      the first entry of every run of equal codes sums the run in
//             FP64 and writes the grid point; run heads are numbered by an
//             exclusive scan of head flags.
// All arithmetic of `spread` rounds each operation separately (no fused
// multiply-add), in the order of the host path (redist.cpp), so both produce
// the same grid points bit for bit.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "nbody.h"
#include "redist.h"
#include "runtime.h"

namespace cvtx {
namespace {

constexpr int kThreads = 256;

// Redistribution functions (reference src/RedistFunc.cpp:35-96), one rounding
// per operation in the order of the C expressions.
__device__ __forceinline__ float redist_fn(int kind, float u) {
	switch (kind) {
	case 0: return u < 0.5f ? 1.f : 0.f;
	case 1: return u <= 1.f ? __fsub_rn(1.f, u) : 0.f;
	case 2:
		return u < 0.5f ? __fsub_rn(1.f, __fmul_rn(u, u))
			: (u < 1.5f ? __fmul_rn(__fmul_rn(0.5f, __fsub_rn(1.f, u)), __fsub_rn(2.f, u)) : 0.f);
	case 3:
		return u < 1.f
			? __fmul_rn(__fmul_rn(0.5f, __fsub_rn(1.f, __fmul_rn(u, u))), __fsub_rn(2.f, u))
			: (u < 2.f ? __fmul_rn(__fmul_rn(__fmul_rn(1.f / 6.f, __fsub_rn(1.f, u)),
				__fsub_rn(2.f, u)), __fsub_rn(3.f, u)) : 0.f);
	default:
		if (u < 1.f) {
			const float a = __fsub_rn(1.f, __fmul_rn(__fmul_rn(2.5f, u), u));
			const float b = __fmul_rn(__fmul_rn(__fmul_rn(1.5f, u), u), u);
			return __fadd_rn(a, b);
		}
		return u < 2.f ? __fmul_rn(__fmul_rn(__fmul_rn(0.5f, __fsub_rn(1.f, u)),
			__fsub_rn(2.f, u)), __fsub_rn(2.f, u)) : 0.f;
	}
}

__device__ __forceinline__ uint64_t d_spread3(uint32_t v) {
	uint64_t x = v & 0x1fffffu;
	x = (x | (x << 32)) & 0x1f00000000ffffull;
	x = (x | (x << 16)) & 0x1f0000ff0000ffull;
	x = (x | (x << 8)) & 0x100f00f00f00f00full;
	x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
	x = (x | (x << 2)) & 0x1249249249249249ull;
	return x;
}
__device__ __forceinline__ uint64_t d_spread2(uint32_t v) {
	uint64_t x = v;
	x = (x | (x << 16)) & 0x0000ffff0000ffffull;
	x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
	x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
	x = (x | (x << 2)) & 0x3333333333333333ull;
	x = (x | (x << 1)) & 0x5555555555555555ull;
	return x;
}

struct SpreadArgs {
	const float* pos;   // dims per particle
	const float* str;   // nc per particle
	int n, dims, nc, radius, S;
	float min[3];
	float gd, rgd;
	int kind;
	uint64_t invalid;   // code of a dropped (zero) contribution
};

__global__ void spread_kernel(const SpreadArgs a, uint64_t* __restrict__ code,
	uint32_t* __restrict__ idx, float* __restrict__ val)
{
	const size_t e = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (e >= size_t(a.n) * size_t(a.S)) return;
	const int i = int(e / size_t(a.S));
	const int s = int(e % size_t(a.S));
	const int w = 2 * a.radius + 1;
	int off[3];
	if (a.dims == 3) { off[0] = s / (w * w); off[1] = (s / w) % w; off[2] = s % w; }
	else { off[0] = s / w; off[1] = s % w; off[2] = 0; }
	float frac = 1.f;
	uint32_t key[3] = {0u, 0u, 0u};
	for (int d = 0; d < a.dims; ++d) {
		const float x = a.pos[size_t(i) * a.dims + d];
		const float t = __fmul_rn(__fsub_rn(x, a.min[d]), a.rgd);
		key[d] = uint32_t(int64_t(roundf(t))) + uint32_t(off[d] - a.radius);
		const float np = __fadd_rn(a.min[d], __fmul_rn(a.gd, float(key[d])));
		const float u = fabsf(__fmul_rn(__fsub_rn(x, np), a.rgd));
		const float f = redist_fn(a.kind, u);
		frac = d == 0 ? f : __fmul_rn(frac, f);
	}
	bool nz = false;
	for (int c = 0; c < a.nc; ++c) {
		const float v = __fmul_rn(a.str[size_t(i) * a.nc + c], frac);
		val[e * a.nc + c] = v;
		nz = nz || v != 0.f;
	}
	const uint64_t cd = a.dims == 3
		? (d_spread3(key[0]) | (d_spread3(key[1]) << 1) | (d_spread3(key[2]) << 2))
		: (d_spread2(key[0]) | (d_spread2(key[1]) << 1));
	code[e] = nz ? cd : a.invalid;
	idx[e] = uint32_t(e);
}

__global__ void head_kernel(const uint64_t* __restrict__ code, size_t m, uint64_t invalid,
	uint32_t* __restrict__ head)
{
	const size_t j = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (j >= m) return;
	head[j] = (code[j] != invalid && (j == 0 || code[j] != code[j - 1])) ? 1u : 0u;
}

__global__ void sum_kernel(const uint64_t* __restrict__ code, const uint32_t* __restrict__ idx,
	const float* __restrict__ val, const uint32_t* __restrict__ head,
	const uint32_t* __restrict__ slot, size_t m, int nc, uint64_t* __restrict__ out_code,
	float* __restrict__ out_val)
{
	const size_t j = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (j >= m || !head[j]) return;
	double acc[3] = {0.0, 0.0, 0.0};
	const uint64_t c = code[j];
	for (size_t q = j; q < m && code[q] == c; ++q)
		for (int k = 0; k < nc; ++k) acc[k] += double(val[size_t(idx[q]) * nc + k]);
	const uint32_t s = slot[j];
	out_code[s] = c;
	for (int k = 0; k < nc; ++k) out_val[size_t(s) * nc + k] = float(acc[k]);
}

inline unsigned blocks_for(size_t m) { return unsigned((m + kThreads - 1) / kThreads); }

}  // namespace

cudaError_t redist_cells_gpu(const RedistGrid& g, int kind, const float* pos, const float* str,
	int n, RedistCells* out, DevBuf* scratch, HostBuf* pinned, cudaStream_t stream)
{
	out->code = nullptr;
	out->vort = nullptr;
	out->n = 0;
	if (n <= 0) return cudaSuccess;
	const int w = 2 * g.radius + 1;
	const int S = g.dims == 3 ? w * w * w : w * w;
	const int nc = g.dims == 3 ? 3 : 1;
	const size_t m = size_t(n) * size_t(S);
	if (m > size_t(0xffffffffu)) return cudaErrorInvalidValue;
	const int key_bits = g.dims * g.bits + 1;   // + the invalid marker bit
	const uint64_t invalid = uint64_t(1) << (g.dims * g.bits);

	// temporary storage size of the sort and the scan
	size_t sort_tmp = 0, scan_tmp = 0;
	cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp,
		static_cast<const uint64_t*>(nullptr), static_cast<uint64_t*>(nullptr),
		static_cast<const uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr), m, 0, key_bits,
		stream);
	if (e == cudaSuccess)
		e = cub::DeviceScan::ExclusiveSum(nullptr, scan_tmp, static_cast<const uint32_t*>(nullptr),
			static_cast<uint32_t*>(nullptr), m, stream);
	if (e != cudaSuccess) return e;
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	const size_t b_pos = al(sizeof(float) * size_t(n) * g.dims);
	const size_t b_str = al(sizeof(float) * size_t(n) * nc);
	const size_t b_code = al(sizeof(uint64_t) * m);
	const size_t b_idx = al(sizeof(uint32_t) * m);
	const size_t b_val = al(sizeof(float) * m * nc);
	const size_t total = b_pos + b_str + 2 * b_code + 2 * b_idx + b_val + 2 * b_idx +
		al(sort_tmp) + al(scan_tmp) + al(sizeof(float) * m * nc) + 256;
	// grow-only: a new allocation only when a call needs more than any before
	e = scratch->ensure(total);
	if (e != cudaSuccess) return e;
	unsigned char* p = static_cast<unsigned char*>(scratch->ptr);
	auto take = [&](size_t b) { unsigned char* r = p; p += b; return r; };
	float* d_pos = reinterpret_cast<float*>(take(b_pos));
	float* d_str = reinterpret_cast<float*>(take(b_str));
	uint64_t* code0 = reinterpret_cast<uint64_t*>(take(b_code));
	uint64_t* code1 = reinterpret_cast<uint64_t*>(take(b_code));
	uint32_t* idx0 = reinterpret_cast<uint32_t*>(take(b_idx));
	uint32_t* idx1 = reinterpret_cast<uint32_t*>(take(b_idx));
	float* val = reinterpret_cast<float*>(take(b_val));
	uint32_t* head = reinterpret_cast<uint32_t*>(take(b_idx));
	uint32_t* slot = reinterpret_cast<uint32_t*>(take(b_idx));
	void* sort_buf = take(al(sort_tmp));
	void* scan_buf = take(al(scan_tmp));
	uint64_t* ocode = code0;   // the unsorted keys are not read after the sort
	float* oval = reinterpret_cast<float*>(take(al(sizeof(float) * m * nc)));

	e = cudaMemcpyAsync(d_pos, pos, sizeof(float) * size_t(n) * g.dims, cudaMemcpyHostToDevice,
		stream);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d_str, str, sizeof(float) * size_t(n) * nc, cudaMemcpyHostToDevice,
			stream);
	if (e != cudaSuccess) return e;
	SpreadArgs a;
	a.pos = d_pos; a.str = d_str; a.n = n; a.dims = g.dims; a.nc = nc; a.radius = g.radius;
	a.S = S; a.gd = g.gd; a.rgd = g.rgd; a.kind = kind; a.invalid = invalid;
	for (int d = 0; d < 3; ++d) a.min[d] = g.min[d];
	spread_kernel<<<blocks_for(m), kThreads, 0, stream>>>(a, code0, idx0, val);
	count_launch();
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	e = cub::DeviceRadixSort::SortPairs(sort_buf, sort_tmp, code0, code1, idx0, idx1, m, 0,
		key_bits, stream);
	if (e != cudaSuccess) return e;
	head_kernel<<<blocks_for(m), kThreads, 0, stream>>>(code1, m, invalid, head);
	count_launch();
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	e = cub::DeviceScan::ExclusiveSum(scan_buf, scan_tmp, head, slot, m, stream);
	if (e != cudaSuccess) return e;
	sum_kernel<<<blocks_for(m), kThreads, 0, stream>>>(code1, idx1, val, head, slot, m, nc,
		ocode, oval);
	count_launch();
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	uint32_t last_slot = 0, last_head = 0;
	e = cudaMemcpyAsync(&last_slot, slot + (m - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost,
		stream);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(&last_head, head + (m - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost,
			stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
	if (e != cudaSuccess) return e;
	const size_t cells = size_t(last_slot) + size_t(last_head);
	if (cells) {
		// the cells go to pinned memory (grow-only), read there by the caller
		const size_t b_c = al(sizeof(uint64_t) * cells);
		e = pinned->ensure(b_c + sizeof(float) * cells * nc);
		if (e != cudaSuccess) return e;
		uint64_t* h_code = static_cast<uint64_t*>(pinned->ptr);
		float* h_vort = reinterpret_cast<float*>(static_cast<unsigned char*>(pinned->ptr) + b_c);
		e = cudaMemcpyAsync(h_code, ocode, sizeof(uint64_t) * cells, cudaMemcpyDeviceToHost,
			stream);
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(h_vort, oval, sizeof(float) * cells * nc, cudaMemcpyDeviceToHost,
				stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
		if (e != cudaSuccess) return e;
		out->code = h_code;
		out->vort = h_vort;
		out->n = cells;
	}
	return e;
}

}  // namespace cvtx
