/* Binning: (tile, item) pairs, emitted in submission order, are stably
 * sorted by tile so that each tile's list keeps primitive order (the
 * reference rasterises primitives strictly one after another,
 * src/pipeline/draw.c:101-122). LSD radix sort with 8-bit digits:
 *   k_radix_global_hist  digit totals of every pass in one read
 *   k_radix_onesweep     one kernel per pass: stable ranks inside each block
 *                        from warp match_any / popc prefix counts, block
 *                        offsets per digit from a decoupled look-back
 * followed by k_tile_ranges, which records each tile's [start, end). */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "kernels.h"
#include "launch.cuh"

namespace srpg {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 8;                       /* per thread */
constexpr int kSortTileItems = kSortThreads * kSortItems;
constexpr int kMaxPasses = 3;                       /* keys up to 24 bits */

/* Digit counts of every pass in one read of the keys (the totals do not
 * depend on the order the passes leave the keys in). */
/* The number of pairs, as counted by setup (at most the scratch's size), or 0
 * once the draw has been aborted. */
__device__ __forceinline__ uint32_t pairCount(const DeviceCounters* ctr, uint32_t cap)
{
	if (ctr->abort) return 0;
	const unsigned long long n = ctr->entries;
	return n < cap ? (uint32_t) n : cap;
}

__global__ void __launch_bounds__(kSortThreads) k_radix_global_hist(const uint32_t* keys, const DeviceCounters* ctr,
                                                                   uint32_t cap, uint32_t passes, uint32_t* ghist)
{
	gridDepSync();
	__shared__ uint32_t h[kMaxPasses][256];
	const uint32_t n = pairCount(ctr, cap);
	if (n == 0) return;
	for (int i = threadIdx.x; i < kMaxPasses * 256; i += kSortThreads) (&h[0][0])[i] = 0;
	__syncthreads();
	for (uint32_t i = blockIdx.x * kSortThreads + threadIdx.x; i < n; i += gridDim.x * kSortThreads) {
		const uint32_t k = keys[i];
		for (uint32_t p = 0; p < passes; ++p) atomicAdd(&h[p][(k >> (8 * p)) & 0xFFu], 1u);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < (int) passes * 256; i += kSortThreads) {
		const uint32_t v = (&h[0][0])[i];
		if (v) atomicAdd(&ghist[i], v);
	}
}

/* Per-digit look-back: predecessor j's word for this digit is at j * 256. */
__device__ __forceinline__ uint32_t lookBackStrided(const uint32_t* status, long long j, uint32_t* errors)
{
	constexpr int W = 8;
	uint32_t acc = 0;
	unsigned spins = 0;
	while (j >= 0) {
		uint32_t v[W];
#pragma unroll
		for (int k = 0; k < W; ++k) v[k] = (j - k >= 0) ? *((volatile const uint32_t*) (status + (j - k) * 256)) : (2u << 30);
#pragma unroll
		for (int k = 0; k < W; ++k) {
			while ((v[k] >> 30) == 0) {
				if (++spins > kSpinLimit) { atomicOr(errors, kErrSpin); return acc; }
				__nanosleep(32);
				v[k] = *((volatile const uint32_t*) (status + (j - k) * 256));
			}
			acc += v[k] & 0x3FFFFFFFu;
			if ((v[k] >> 30) == 2) return acc;
		}
		j -= W;
	}
	return acc;
}

/* One stable LSD pass (OneSweep style). Blocks take 2048 consecutive keys in
 * ticket order; ranks inside the block come from warp match_any / popc prefix
 * counts over rounds that follow input order; each block publishes its 256
 * digit counts and walks back over its predecessors' (decoupled look-back,
 * one thread per digit) to find where its run of each digit starts. */
__global__ void __launch_bounds__(kSortThreads) k_radix_onesweep(const uint32_t* keysIn, const uint32_t* valsIn,
                                                                const DeviceCounters* ctr, uint32_t cap,
                                                                uint32_t shift, const uint32_t* ghistPass,
                                                                uint32_t* status, uint32_t* ticket, uint32_t* errors,
                                                                uint32_t* keysOut, uint32_t* valsOut)
{
	gridDepSync();
	/* the grid is sized for the scratch; blocks past the real count leave at
	 * once (their successors, which would look back at them, leave too) */
	const uint32_t n = pairCount(ctr, cap);
	if ((unsigned long long) blockIdx.x * kSortTileItems >= n) return;
	__shared__ uint32_t cnt[kSortWarps][256];
	__shared__ uint32_t digitBase[256];
	__shared__ uint32_t digitStart[256];
	__shared__ uint32_t sBlock;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (threadIdx.x == 0) sBlock = atomicAdd(ticket, 1u);
	for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads) (&cnt[0][0])[i] = 0;
	/* exclusive scan of the pass's digit totals (Hillis-Steele in shared memory) */
	digitStart[threadIdx.x] = ghistPass[threadIdx.x];
	__syncthreads();
	for (int o = 1; o < 256; o <<= 1) {
		const uint32_t v = threadIdx.x >= o ? digitStart[threadIdx.x - o] : 0u;
		__syncthreads();
		digitStart[threadIdx.x] += v;
		__syncthreads();
	}
	const uint32_t blk = sBlock;
	const uint32_t base = blk * kSortTileItems + warp * (32 * kSortItems);
	const uint32_t ltMask = (1u << lane) - 1u;
	uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
	for (int r = 0; r < kSortItems; ++r) {
		const uint32_t i = base + r * 32 + lane;
		const bool valid = i < n;
		key[r] = valid ? keysIn[i] : 0u;
		val[r] = valid ? valsIn[i] : 0u;
		const uint32_t d = (key[r] >> shift) & 0xFFu;
		const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 256u + lane);
		const uint32_t before = valid ? cnt[warp][d] : 0u;
		__syncwarp();
		if (valid && lane == __ffs(peers) - 1) cnt[warp][d] = before + __popc(peers);
		__syncwarp();
		rank[r] = valid ? before + __popc(peers & ltMask) : 0xFFFFFFFFu;
	}
	__syncthreads();
	{
		/* thread d: exclusive prefix over warps, block total, look-back */
		const int d = threadIdx.x;
		uint32_t run = 0;
#pragma unroll
		for (int w = 0; w < kSortWarps; ++w) { const uint32_t t = cnt[w][d]; cnt[w][d] = run; run += t; }
		uint32_t* st = status + (size_t) blk * 256 + d;
		uint32_t prefix = 0;
		if (blk == 0) {
			atomicExch(st, (2u << 30) | run);
		} else {
			atomicExch(st, (1u << 30) | run);
			prefix = lookBackStrided(status + d, (long long) blk - 1, errors);
			atomicExch(st, (2u << 30) | (prefix + run));
		}
		/* start of digit d in the output: all smaller digits, then earlier blocks */
		digitBase[d] = digitStart[d] - ghistPass[d] + prefix;
	}
	__syncthreads();
#pragma unroll
	for (int r = 0; r < kSortItems; ++r) {
		if (rank[r] == 0xFFFFFFFFu) continue;
		const uint32_t d = (key[r] >> shift) & 0xFFu;
		const uint32_t pos = digitBase[d] + cnt[warp][d] + rank[r];
		keysOut[pos] = key[r];
		valsOut[pos] = val[r];
	}
}

__global__ void k_tile_ranges(const uint32_t* keys, const DeviceCounters* ctr, uint32_t cap, uint32_t numTiles,
                              uint32_t* start, uint32_t* end)
{
	gridDepSync();
	const uint32_t n = pairCount(ctr, cap);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const uint32_t k = keys[i];
		if (k >= numTiles) continue;
		if (i == 0 || keys[i - 1] != k) start[k] = i;
		if (i == n - 1 || keys[i + 1] != k) end[k] = i + 1;
	}
}

static uint32_t sortBlocks(uint32_t n) { return (n + kSortTileItems - 1) / kSortTileItems; }

/* scratch words: global histograms, per-pass look-back status, tickets */
size_t sortHistWords(uint32_t n) { return (size_t) kMaxPasses * 256 + (size_t) kMaxPasses * 256 * (sortBlocks(n) + 1) + 8; }

size_t sortPartialWords(uint32_t) { return 8; }

void sortEntries(const DrawParams& P, uint32_t keyBits, uint32_t* keysAlt, uint32_t* valsAlt,
                 uint32_t* hist, uint32_t*, uint32_t** keysOut, uint32_t** valsOut, cudaStream_t s)
{
	uint32_t* kin = P.keys;
	uint32_t* vin = P.vals;
	uint32_t* kout = keysAlt;
	uint32_t* vout = valsAlt;
	const uint32_t cap = P.entryCap;
	const uint32_t nb = sortBlocks(cap);
	const uint32_t passes = (keyBits + 7) / 8;
	if (cap > 0 && passes) {
		uint32_t* ghist = hist;
		uint32_t* tickets = hist + kMaxPasses * 256;
		uint32_t* status = tickets + 8;
		cudaMemsetAsync(hist, 0, sortHistWords(cap) * 4, s);
		const uint32_t hb = nb < 152u * 4u ? nb : 152u * 4u;
		pdlLaunch(k_radix_global_hist, hb, kSortThreads, 0, s, kin, P.ctr, cap, passes, ghist);
		for (uint32_t p = 0; p < passes; ++p) {
			pdlLaunch(k_radix_onesweep, nb, kSortThreads, 0, s, kin, vin, P.ctr, cap, 8 * p, ghist + 256 * p,
			                                            status + (size_t) p * 256 * nb, tickets + p, &P.ctr->errors,
			                                            kout, vout);
			uint32_t* t = kin; kin = kout; kout = t;
			t = vin; vin = vout; vout = t;
		}
	}
	*keysOut = kin;
	*valsOut = vin;
}

void launchTileRanges(const DrawParams& P, const uint32_t* keys, uint32_t numTiles, cudaStream_t s)
{
	const uint32_t cap = P.entryCap;
	if (!cap) return;
	const uint32_t blocks = (cap + 255) / 256 < 152u * 16u ? (cap + 255) / 256 : 152u * 16u;
	pdlLaunch(k_tile_ranges, blocks, 256, 0, s, keys, P.ctr, cap, numTiles, P.tileStart, P.tileEnd);
}

}  // namespace srpg
