/* Binning: (tile, item) pairs, emitted in submission order, are stably
 * sorted by tile so that each tile's list keeps primitive order (the
 * reference rasterises primitives strictly one after another,
 * src/pipeline/draw.c:101-122). LSD radix sort with 8-bit digits:
 *   k_radix_hist    per-block digit histograms, stored digit-major
 *   k_scan_*        exclusive scan of the histograms (global digit offsets)
 *   k_radix_scatter stable ranks inside each block from warp match_any /
 *                   popc prefix counts, then the scatter
 * followed by k_tile_ranges, which records each tile's [start, end). */
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace srpg {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 8;                       /* per thread */
constexpr int kSortTileItems = kSortThreads * kSortItems;
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanChunk = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint32_t* keys, uint32_t n, uint32_t shift,
                                                            uint32_t* hist, uint32_t nBlocks)
{
	__shared__ uint32_t h[256];
	h[threadIdx.x] = 0;
	__syncthreads();
	const uint32_t base = blockIdx.x * kSortTileItems;
	for (int r = 0; r < kSortItems; ++r) {
		const uint32_t i = base + r * kSortThreads + threadIdx.x;
		if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFFu], 1u);
	}
	__syncthreads();
	hist[threadIdx.x * nBlocks + blockIdx.x] = h[threadIdx.x];
}

/* Block-wide exclusive scan of kScanItems values per thread (in order). */
__device__ __forceinline__ uint32_t blockScanExclusive(uint32_t v[kScanItems], uint32_t* sWarp)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t local = 0;
#pragma unroll
	for (int k = 0; k < kScanItems; ++k) { const uint32_t t = v[k]; v[k] = local; local += t; }
	uint32_t incl = local;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
		if (lane >= o) incl += y;
	}
	if (lane == 31) sWarp[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		uint32_t w = lane < kScanThreads / 32 ? sWarp[lane] : 0u;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
			if (lane >= o) w += y;
		}
		if (lane < kScanThreads / 32) sWarp[lane] = w;
	}
	__syncthreads();
	const uint32_t off = (warp ? sWarp[warp - 1] : 0u) + incl - local;
	const uint32_t total = sWarp[kScanThreads / 32 - 1];
#pragma unroll
	for (int k = 0; k < kScanItems; ++k) v[k] += off;
	__syncthreads();
	return total;
}

/* Pass 1: scan each chunk in place, record the chunk total. */
__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(uint32_t* data, uint32_t n, uint32_t* partials)
{
	__shared__ uint32_t sWarp[kScanThreads / 32];
	const uint32_t base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
	uint32_t v[kScanItems];
#pragma unroll
	for (int k = 0; k < kScanItems; ++k) v[k] = base + k < n ? data[base + k] : 0u;
	const uint32_t total = blockScanExclusive(v, sWarp);
#pragma unroll
	for (int k = 0; k < kScanItems; ++k) if (base + k < n) data[base + k] = v[k];
	if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

/* Pass 2: one block scans the chunk totals, kScanChunk at a time with a
 * running carry. */
__global__ void __launch_bounds__(kScanThreads) k_scan_partials(uint32_t* partials, uint32_t n)
{
	__shared__ uint32_t sWarp[kScanThreads / 32];
	uint32_t carry = 0;
	for (uint32_t off = 0; off < n; off += kScanChunk) {
		const uint32_t base = off + threadIdx.x * kScanItems;
		uint32_t v[kScanItems];
#pragma unroll
		for (int k = 0; k < kScanItems; ++k) v[k] = base + k < n ? partials[base + k] : 0u;
		const uint32_t total = blockScanExclusive(v, sWarp);
#pragma unroll
		for (int k = 0; k < kScanItems; ++k) if (base + k < n) partials[base + k] = v[k] + carry;
		carry += total;
	}
}

/* Pass 3: add each chunk's offset. */
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(uint32_t* data, uint32_t n, const uint32_t* partials)
{
	const uint32_t off = partials[blockIdx.x];
	const uint32_t base = blockIdx.x * kScanChunk;
	for (int k = threadIdx.x; k < kScanChunk; k += kScanThreads)
		if (base + k < n) data[base + k] += off;
}

__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint32_t* keysIn, const uint32_t* valsIn, uint32_t n,
                                                               uint32_t shift, const uint32_t* offsets, uint32_t nBlocks,
                                                               uint32_t* keysOut, uint32_t* valsOut)
{
	__shared__ uint32_t cnt[kSortWarps][256];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads) (&cnt[0][0])[i] = 0;
	__syncthreads();
	const uint32_t base = blockIdx.x * kSortTileItems + warp * (32 * kSortItems);
	const uint32_t ltMask = (1u << lane) - 1u;
	uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
	for (int r = 0; r < kSortItems; ++r) {
		const uint32_t i = base + r * 32 + lane;
		const bool valid = i < n;
		key[r] = valid ? keysIn[i] : 0u;
		val[r] = valid ? valsIn[i] : 0u;
		const uint32_t d = (key[r] >> shift) & 0xFFu;
		/* lanes holding the same digit in this round, in lane (= input) order */
		const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 256u + lane);
		const uint32_t before = valid ? cnt[warp][d] : 0u;
		__syncwarp();
		if (valid && lane == __ffs(peers) - 1) cnt[warp][d] = before + __popc(peers);
		__syncwarp();
		rank[r] = valid ? before + __popc(peers & ltMask) : 0xFFFFFFFFu;
	}
	__syncthreads();
	/* per digit, exclusive prefix over warps: earlier warps hold earlier items */
	{
		const int d = threadIdx.x;
		uint32_t run = 0;
#pragma unroll
		for (int w = 0; w < kSortWarps; ++w) { const uint32_t t = cnt[w][d]; cnt[w][d] = run; run += t; }
	}
	__syncthreads();
#pragma unroll
	for (int r = 0; r < kSortItems; ++r) {
		if (rank[r] == 0xFFFFFFFFu) continue;
		const uint32_t d = (key[r] >> shift) & 0xFFu;
		const uint32_t pos = offsets[d * nBlocks + blockIdx.x] + cnt[warp][d] + rank[r];
		keysOut[pos] = key[r];
		valsOut[pos] = val[r];
	}
}

__global__ void k_tile_ranges(const uint32_t* keys, uint32_t n, uint32_t numTiles, uint32_t* start, uint32_t* end)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const uint32_t k = keys[i];
	if (k >= numTiles) return;
	if (i == 0 || keys[i - 1] != k) start[k] = i;
	if (i == n - 1 || keys[i + 1] != k) end[k] = i + 1;
}

static uint32_t sortBlocks(uint32_t n) { return (n + kSortTileItems - 1) / kSortTileItems; }

size_t sortHistWords(uint32_t n) { return (size_t) 256 * (sortBlocks(n) ? sortBlocks(n) : 1); }

size_t sortPartialWords(uint32_t n)
{
	const size_t m = sortHistWords(n);
	return (m + kScanChunk - 1) / kScanChunk + 1;
}

static void scanExclusive(uint32_t* data, uint32_t n, uint32_t* partials, cudaStream_t s)
{
	const uint32_t chunks = (n + kScanChunk - 1) / kScanChunk;
	k_scan_chunks<<<chunks, kScanThreads, 0, s>>>(data, n, partials);
	if (chunks > 1) {
		k_scan_partials<<<1, kScanThreads, 0, s>>>(partials, chunks);
		k_scan_apply<<<chunks, kScanThreads, 0, s>>>(data, n, partials);
	}
}

void sortEntries(const DrawParams& P, uint32_t n, uint32_t keyBits, uint32_t* keysAlt, uint32_t* valsAlt,
                 uint32_t* hist, uint32_t* partials, uint32_t** keysOut, uint32_t** valsOut, cudaStream_t s)
{
	uint32_t* kin = P.keys;
	uint32_t* vin = P.vals;
	uint32_t* kout = keysAlt;
	uint32_t* vout = valsAlt;
	const uint32_t nb = sortBlocks(n);
	if (n > 1) {
		for (uint32_t shift = 0; shift < keyBits; shift += 8) {
			k_radix_hist<<<nb, kSortThreads, 0, s>>>(kin, n, shift, hist, nb);
			scanExclusive(hist, 256 * nb, partials, s);
			k_radix_scatter<<<nb, kSortThreads, 0, s>>>(kin, vin, n, shift, hist, nb, kout, vout);
			uint32_t* t = kin; kin = kout; kout = t;
			t = vin; vin = vout; vout = t;
		}
	}
	*keysOut = kin;
	*valsOut = vin;
}

void launchTileRanges(const DrawParams& P, const uint32_t* keys, uint32_t n, uint32_t numTiles, cudaStream_t s)
{
	if (!n) return;
	k_tile_ranges<<<(n + 255) / 256, 256, 0, s>>>(keys, n, numTiles, P.tileStart, P.tileEnd);
}

}  // namespace srpg
