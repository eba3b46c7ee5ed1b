// common.cuh -- device primitives shared by the all-pairs kernels (sm_103a).
//
// * Source tiles are moved global -> shared by the bulk-copy engine
//   (cp.async.bulk, 1-D, no tensor map) and paced by one mbarrier per stage.
//   Every wait on an mbarrier is bounded by a wall-clock deadline read from
//   %globaltimer; on expiry the kernel records an error code and returns.
// * Per-target sums are compensated: FP32 partials over one source tile are
//   folded into a (hi, lo) pair with Knuth's TwoSum, so the cross-tile sum
//   carries roughly twice the FP32 mantissa.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cvtx {

// Error codes written to the device error word (host reads it after a call).
enum : unsigned {
	kErrNone = 0u,
	kErrPipelineTimeout = 1u,   // an mbarrier wait exceeded its deadline
	kErrDrainTimeout = 2u,      // draining in-flight copies after an error timed out
	kErrBadCopy = 4u,           // a bulk copy had a misaligned address or size (skipped)
	kErrBadLaunch = 8u,         // launch shape or shared-memory base not as the kernel expects
	kErrBadWork = 16u,          // a work item out of range (skipped)
};

// Deadline for one mbarrier wait: source tiles land in microseconds, so two
// seconds only trips when something is wrong.
constexpr unsigned long long kWaitDeadlineNs = 2000000000ull;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
		:: "r"(smem_addr(bar)), "r"(count) : "memory");
}

// Make barrier initialisation visible to the async (bulk-copy) proxy.
__device__ __forceinline__ void mbar_init_fence() {
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy writes into the same buffer (stage refill after reuse).
__device__ __forceinline__ void fence_proxy_async() {
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
	asm volatile("{\n\t.reg .b64 st;\n\t"
		"mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
		:: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// 1-D bulk copy global -> shared, completion signalled on `bar` as bytes.
// Requirements (checked by callers): both addresses 16-byte aligned and
// `bytes` a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst_smem, const void* src_gmem,
	uint32_t bytes, uint64_t* bar) {
	asm volatile(
		"cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes"
		" [%0], [%1], %2, [%3];"
		:: "r"(smem_addr(dst_smem)), "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
		: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
	return ok != 0u;
}

// Wait for phase `parity` of `bar` for at most `limit_ns`. Returns false on
// expiry.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity,
	unsigned long long limit_ns) {
	if (mbar_try_wait(bar, parity)) return true;
	const unsigned long long t0 = globaltimer_ns();
	while (true) {
		if (mbar_try_wait(bar, parity)) return true;
		if (globaltimer_ns() - t0 > limit_ns) return false;
	}
}

// Bounded wait for phase `parity` of `bar`. Returns false on deadline expiry.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
	return mbar_wait_for(bar, parity, kWaitDeadlineNs);
}

__device__ __forceinline__ float rsqrt_approx(float x) {
	float y;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

// 2^x and 1/x from the special-function unit (a few ulp; ftz).
__device__ __forceinline__ float ex2_approx(float x) {
	float y;
	asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}
// max(a, b, c), NaN if any input is NaN (three-input form, sm_100 and up).
__device__ __forceinline__ float max3_nan(float a, float b, float c) {
	float y;
	asm("max.NaN.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(a), "f"(b), "f"(c));
	return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
	float y;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

// rsqrt with one Newton step, y (1.5 - 0.5 x y^2): about half an ulp, for
// kernels whose per-pair weights are high powers of 1/r (errors triple in 1/r^3).
__device__ __forceinline__ float rsqrt_refined(float x) {
	const float y = rsqrt_approx(x);
	const float h = x * y;
	return y * fmaf(-0.5f * h, y, 1.5f);
}

// Knuth TwoSum fold of an FP32 tile partial `p` into the pair (hi, lo).
__device__ __forceinline__ void fold_twosum(float& hi, float& lo, float p) {
	const float s = __fadd_rn(hi, p);
	const float bp = __fsub_rn(s, hi);
	const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
	hi = s;
	lo = __fadd_rn(lo, err);
}

}  // namespace cvtx
