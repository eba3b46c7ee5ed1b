// pack.cu -- repack caller records that are already in device memory into
// the float4 records the all-pairs kernels read (layouts in nbody.h).
// Memory-bound elementwise kernels: each thread moves one record.
#include "nbody.h"

namespace cvtx {
namespace {

constexpr int kThreads = 256;

// cvtx_P3D: 7 floats (coord[3], vorticity[3], volume), 28-byte stride.
__global__ void pack_p3d_kernel(const float* __restrict__ aos, int n, float4* __restrict__ out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float* r = aos + size_t(i) * 7;
	out[2 * size_t(i)] = make_float4(r[0], r[1], r[2], r[6]);
	out[2 * size_t(i) + 1] = make_float4(r[3], r[4], r[5], 0.f);
}
// cvtx_F3D: 7 floats (start[3], end[3], strength).
__global__ void pack_f3d_kernel(const float* __restrict__ aos, int n, float4* __restrict__ out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float* r = aos + size_t(i) * 7;
	out[2 * size_t(i)] = make_float4(r[0], r[1], r[2], r[6]);
	out[2 * size_t(i) + 1] = make_float4(r[3], r[4], r[5], 0.f);
}
// cvtx_P2D: 4 floats (coord[2], vorticity, area) -- already the record layout.
__global__ void pack_p2d_kernel(const float* __restrict__ aos, int n, float4* __restrict__ out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float* r = aos + size_t(i) * 4;
	out[i] = make_float4(r[0], r[1], r[2], r[3]);
}
__global__ void pack_v3_kernel(const float* __restrict__ v, int n, float4* __restrict__ out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float* r = v + size_t(i) * 3;
	out[i] = make_float4(r[0], r[1], r[2], 0.f);
}
__global__ void pack_v2_kernel(const float* __restrict__ v, int n, float4* __restrict__ out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float* r = v + size_t(i) * 2;
	out[i] = make_float4(r[0], r[1], 0.f, 0.f);
}
// Gather through an array of record pointers that the device can dereference.
__global__ void gather_p3d_kernel(const float* const* __restrict__ ptrs, int n,
	float4* __restrict__ out) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float* r = ptrs[i];
	out[2 * size_t(i)] = make_float4(r[0], r[1], r[2], r[6]);
	out[2 * size_t(i) + 1] = make_float4(r[3], r[4], r[5], 0.f);
}

inline int blocks(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

cudaError_t pack_p3d(const void* aos28, int n, float4* out, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	pack_p3d_kernel<<<blocks(n), kThreads, 0, s>>>(static_cast<const float*>(aos28), n, out);
	count_launch();
	return cudaGetLastError();
}
cudaError_t pack_f3d(const void* aos28, int n, float4* out, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	pack_f3d_kernel<<<blocks(n), kThreads, 0, s>>>(static_cast<const float*>(aos28), n, out);
	count_launch();
	return cudaGetLastError();
}
cudaError_t pack_p2d(const void* aos16, int n, float4* out, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	pack_p2d_kernel<<<blocks(n), kThreads, 0, s>>>(static_cast<const float*>(aos16), n, out);
	count_launch();
	return cudaGetLastError();
}
cudaError_t pack_v3(const void* v12, int n, float4* out, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	pack_v3_kernel<<<blocks(n), kThreads, 0, s>>>(static_cast<const float*>(v12), n, out);
	count_launch();
	return cudaGetLastError();
}
cudaError_t pack_v2(const void* v8, int n, float4* out, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	pack_v2_kernel<<<blocks(n), kThreads, 0, s>>>(static_cast<const float*>(v8), n, out);
	count_launch();
	return cudaGetLastError();
}
cudaError_t gather_p3d(const void* const* ptrs, int n, float4* out, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	gather_p3d_kernel<<<blocks(n), kThreads, 0, s>>>(
		reinterpret_cast<const float* const*>(ptrs), n, out);
	count_launch();
	return cudaGetLastError();
}

}  // namespace cvtx
