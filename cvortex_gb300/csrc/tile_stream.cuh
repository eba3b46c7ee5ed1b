// tile_stream.cuh -- stream a contiguous range of source records through
// shared memory in tiles, double-buffered, with bulk copies paced by
// mbarriers. One thread (thread 0) issues copies; every thread waits on the
// stage's mbarrier with a bounded wait, processes the tile, then the CTA
// synchronises before the stage is refilled.
//
// A source record is REC float4s (16 * REC bytes). The global record array
// must be 16-byte aligned (device allocations are 256-byte aligned).
#pragma once
#include "common.cuh"

namespace cvtx {

template <int REC, int TILE, int STAGES>
struct TileStream {
	static constexpr size_t kTileBytes = size_t(TILE) * REC * 16;
	static constexpr size_t kSmemBytes = STAGES * kTileBytes + STAGES * sizeof(uint64_t);

	// Initialise the stage barriers (once per CTA, all threads must call it).
	// Returns false, with kErrBadLaunch in the error word, if `smem` is not
	// 16-byte aligned (the caller must then return).
	__device__ __forceinline__ static bool init(unsigned char* smem, unsigned* err) {
		if (__syncthreads_or((smem_addr(smem) & 15u) != 0u)) {
			if (threadIdx.x == 0) atomicOr(err, kErrBadLaunch);
			return false;
		}
		uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * kTileBytes);
		if (threadIdx.x == 0) {
			for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1u);
			mbar_init_fence();
		}
		__syncthreads();
		return true;
	}

	// `smem` must be 16-byte aligned and kSmemBytes long. `fn(tile, count)` is
	// called once per tile by every thread with a pointer to the staged
	// records and the number of valid records (== TILE except for the last).
	// Returns false (after draining in-flight copies) if a wait expired; the
	// caller must then return without writing results.
	template <class Fn>
	__device__ __forceinline__ static bool run(unsigned char* smem,
		const float4* __restrict__ src, int s_begin, int n_s, unsigned* err, Fn&& fn)
	{
		if (!init(smem, err)) return false;
		unsigned tcount = 0;
		return run_continue(smem, src, s_begin, n_s, err, tcount, fn);
	}

	// As run(), on barriers initialised earlier by init(): `tcount` counts the
	// tiles this CTA has streamed before (it selects stage and phase parity)
	// and is advanced by the tiles streamed now. Lets a persistent CTA stream
	// many source ranges without re-initialising its barriers.
	template <class Fn>
	__device__ __forceinline__ static bool run_continue(unsigned char* smem,
		const float4* __restrict__ src, int s_begin, int n_s, unsigned* err, unsigned& tcount,
		Fn&& fn)
	{
		float4* tiles = reinterpret_cast<float4*>(smem);
		uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * kTileBytes);
		const int n_tiles = (n_s + TILE - 1) / TILE;
		const unsigned base = tcount;
		if (threadIdx.x == 0) {
			// stages may hold records of an earlier range read through the
			// generic proxy; order those reads before the bulk-copy writes
			fence_proxy_async();
			const int pro = n_tiles < STAGES ? n_tiles : STAGES;
			for (int t = 0; t < pro; ++t) issue(tiles, bars, src, s_begin, n_s, t, base, err);
		}
		for (int it = 0; it < n_tiles; ++it) {
			const unsigned g = base + unsigned(it);
			const int stage = int(g % STAGES);
			const bool ok = mbar_wait_bounded(&bars[stage], (g / STAGES) & 1u);
			if (__syncthreads_or(!ok)) {
				if (threadIdx.x == 0) {
					atomicOr(err, kErrPipelineTimeout);
					const int last = (it + STAGES < n_tiles) ? it + STAGES : n_tiles;
					for (int t = it; t < last; ++t) {
						const unsigned gt = base + unsigned(t);
						if (!mbar_wait_bounded(&bars[gt % STAGES], (gt / STAGES) & 1u))
							atomicOr(err, kErrDrainTimeout);
					}
				}
				__syncthreads();
				return false;
			}
			const int rem = n_s - it * TILE;
			fn(tiles + size_t(stage) * TILE * REC, rem < TILE ? rem : TILE);
			__syncthreads();
			if (threadIdx.x == 0 && it + STAGES < n_tiles) {
				fence_proxy_async();
				issue(tiles, bars, src, s_begin, n_s, it + STAGES, base, err);
			}
		}
		tcount = base + unsigned(n_tiles);
		return true;
	}

 private:
	// A copy whose addresses or size break the bulk-copy rules (16-byte
	// aligned addresses, size a positive multiple of 16) is not issued: the
	// stage barrier is completed by a plain arrival instead and the error
	// word records it, so the kernel finishes and the host reports the error.
	__device__ __forceinline__ static void issue(float4* tiles, uint64_t* bars,
		const float4* __restrict__ src, int s_begin, int n_s, int t, unsigned base, unsigned* err)
	{
		const int stage = int((base + unsigned(t)) % STAGES);
		const int rem = n_s - t * TILE;
		const int cnt = rem < TILE ? rem : TILE;
		const uint32_t bytes = uint32_t(cnt) * REC * 16u;
		float4* dst = tiles + size_t(stage) * TILE * REC;
		const float4* from = src + (size_t(s_begin) + size_t(t) * TILE) * REC;
		const bool bad = cnt <= 0 || cnt > TILE || (smem_addr(dst) & 15u) != 0u ||
			(reinterpret_cast<uintptr_t>(from) & 15u) != 0u;
		if (bad) {
			atomicOr(err, kErrBadCopy);
			mbar_arrive_expect_tx(&bars[stage], 0u);
			return;
		}
		mbar_arrive_expect_tx(&bars[stage], bytes);
		bulk_copy_g2s(dst, from, bytes, &bars[stage]);
	}
};

}  // namespace cvtx
