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

	// `smem` must be 16-byte aligned and kSmemBytes long. `fn(tile, count)` is
	// called once per tile by every thread with a pointer to the staged
	// records and the number of valid records (== TILE except for the last).
	// Returns false (after draining in-flight copies) if a wait expired; the
	// caller must then return without writing results.
	template <class Fn>
	__device__ __forceinline__ static bool run(unsigned char* smem,
		const float4* __restrict__ src, int s_begin, int n_s, unsigned* err, Fn&& fn)
	{
		float4* tiles = reinterpret_cast<float4*>(smem);
		uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * kTileBytes);
		const int n_tiles = (n_s + TILE - 1) / TILE;
		if (threadIdx.x == 0) {
			for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1u);
			mbar_init_fence();
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			const int pro = n_tiles < STAGES ? n_tiles : STAGES;
			for (int t = 0; t < pro; ++t) issue(tiles, bars, src, s_begin, n_s, t);
		}
		for (int it = 0; it < n_tiles; ++it) {
			const int stage = it % STAGES;
			const bool ok = mbar_wait_bounded(&bars[stage], uint32_t((it / STAGES) & 1));
			if (__syncthreads_or(!ok)) {
				if (threadIdx.x == 0) {
					atomicOr(err, kErrPipelineTimeout);
					const int last = (it + STAGES < n_tiles) ? it + STAGES : n_tiles;
					for (int t = it; t < last; ++t)
						if (!mbar_wait_bounded(&bars[t % STAGES], uint32_t((t / STAGES) & 1)))
							atomicOr(err, kErrDrainTimeout);
				}
				__syncthreads();
				return false;
			}
			const int rem = n_s - it * TILE;
			fn(tiles + size_t(stage) * TILE * REC, rem < TILE ? rem : TILE);
			__syncthreads();
			if (threadIdx.x == 0 && it + STAGES < n_tiles) {
				fence_proxy_async();
				issue(tiles, bars, src, s_begin, n_s, it + STAGES);
			}
		}
		return true;
	}

 private:
	__device__ __forceinline__ static void issue(float4* tiles, uint64_t* bars,
		const float4* __restrict__ src, int s_begin, int n_s, int t)
	{
		const int stage = t % STAGES;
		const int rem = n_s - t * TILE;
		const int cnt = rem < TILE ? rem : TILE;
		const uint32_t bytes = uint32_t(cnt) * REC * 16u;
		mbar_arrive_expect_tx(&bars[stage], bytes);
		bulk_copy_g2s(tiles + size_t(stage) * TILE * REC,
			src + (size_t(s_begin) + size_t(t) * TILE) * REC, bytes, &bars[stage]);
	}
};

}  // namespace cvtx
