// advance.cu -- device-resident forward-Euler update of particle state.
//
// The step either side of the all-pairs path: after the induced velocity (and,
// for 3D particles, the vorticity rate) has been computed on the device, move
// the particles without a host round trip:
//   P3D record (x, y, z, vol), (a_x, a_y, a_z, 0):  x += dt u,  a += dt da/dt
//   P2D record (x, y, Gamma, area):                  x += dt u
//   point (x, y, z, 0):                              x += dt u
// The reference leaves time integration to its callers (all state lives in
// caller arrays); this is the update a caller of the reference applies between
// two cvtx_*_M2M_vel / cvtx_P3D_M2M_dvort calls. HBM-bound: one thread per
// record, float4 loads and stores.
#include "nbody.h"

namespace cvtx {
namespace {

constexpr int kThreads = 256;

__global__ void advance_p3d_kernel(float4* __restrict__ rec, int n,
	const float* __restrict__ vel, const float* __restrict__ dvort, float dt)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	float4 p = rec[2 * size_t(i)];
	const float* u = vel + 3 * size_t(i);
	p.x = fmaf(dt, u[0], p.x);
	p.y = fmaf(dt, u[1], p.y);
	p.z = fmaf(dt, u[2], p.z);
	rec[2 * size_t(i)] = p;
	if (dvort) {
		float4 a = rec[2 * size_t(i) + 1];
		const float* w = dvort + 3 * size_t(i);
		a.x = fmaf(dt, w[0], a.x);
		a.y = fmaf(dt, w[1], a.y);
		a.z = fmaf(dt, w[2], a.z);
		rec[2 * size_t(i) + 1] = a;
	}
}

__global__ void advance_p2d_kernel(float4* __restrict__ rec, int n,
	const float* __restrict__ vel, float dt)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	float4 p = rec[i];
	p.x = fmaf(dt, vel[2 * size_t(i)], p.x);
	p.y = fmaf(dt, vel[2 * size_t(i) + 1], p.y);
	rec[i] = p;
}

__global__ void advance_points_kernel(float4* __restrict__ pts, int n,
	const float* __restrict__ vel, float dt)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	float4 p = pts[i];
	const float* u = vel + 3 * size_t(i);
	p.x = fmaf(dt, u[0], p.x);
	p.y = fmaf(dt, u[1], p.y);
	p.z = fmaf(dt, u[2], p.z);
	pts[i] = p;
}

inline int blocks(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

cudaError_t advance_p3d(float4* rec, int n, const float* vel, const float* dvort, float dt,
	cudaStream_t s)
{
	if (n <= 0) return cudaSuccess;
	advance_p3d_kernel<<<blocks(n), kThreads, 0, s>>>(rec, n, vel, dvort, dt);
	count_launch();
	return cudaGetLastError();
}

cudaError_t advance_p2d(float4* rec, int n, const float* vel, float dt, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	advance_p2d_kernel<<<blocks(n), kThreads, 0, s>>>(rec, n, vel, dt);
	count_launch();
	return cudaGetLastError();
}

cudaError_t advance_points(float4* pts, int n, const float* vel, float dt, cudaStream_t s) {
	if (n <= 0) return cudaSuccess;
	advance_points_kernel<<<blocks(n), kThreads, 0, s>>>(pts, n, vel, dt);
	count_launch();
	return cudaGetLastError();
}

}  // namespace cvtx
