/* Per-tile rasterisation: visibility resolve and deferred shading.
 *
 * One warp owns one 8x8 tile; lane l owns pixels l and l + 32 of it. The
 * tile's items (triangles, points or line fragments, already in submission
 * order) are taken 32 at a time:
 *   phase 1  lane j evaluates item j over the tile -- for a triangle the
 *            reference's incremental barycentrics (exact chain, see chain.h)
 *            and the top-left test -- leaving a 64-bit coverage mask and the
 *            per-pixel depths in shared memory;
 *   phase 2  each lane walks, for its own pixels, the covering items in order
 *            and applies the stencil test, the depth test and the stencil
 *            operations exactly as the reference's emitFragment does
 *            (src/raster/fragment.c:63-125), remembering the last item that
 *            reached the colour write.
 * Because srp has no blending and a shader that does not write fragDepth
 * cannot influence depth or stencil, the colour of a pixel is the shader
 * output of that last item; k_shade evaluates it once per pixel afterwards.
 * Shaders that write fragDepth take the in-order path (k_resolve with
 * LATE_FS), which shades every fragment in phase 2. */
#include "raster_common.cuh"

namespace srpg {

/* The warp tiles of the depth and winner planes that the TMA variant of the
 * light-tile resolve stages in shared memory; nothing in the other variants,
 * whose occupancy the extra shared memory would lower. */
template <bool TMA> struct ResolveTiles {
	__align__(128) float depth[kResolveWarps][64];
	__align__(128) int32_t winner[kResolveWarps][64];
	unsigned long long bar[kResolveWarps];
};
template <> struct ResolveTiles<false> {};

/* TMA: the variant for single draws whose tiles move by TMA (DrawParams::tma
 * selects which copies). */
template <int KIND, int LATE_FS, bool MULTI = false, bool TMA = false>
__global__ void __launch_bounds__(kResolveWarps * 32, MULTI ? 8 : 1) k_resolve(const __grid_constant__ DrawParams P,
                                                                              const uint32_t* vals, uint32_t numTiles)
{
	gridDepSync();
	constexpr int kResolveChunk = MULTI ? kResolveChunkMulti : 32;
	__shared__ unsigned long long sMask[kResolveWarps][32];
	__shared__ uint32_t sItem[kResolveWarps][32];
	__shared__ uint32_t sFlag[kResolveWarps][32];
	__shared__ float sDep[kResolveWarps][kResolveChunk][kDepRow];
	__shared__ TriRaster sRec[KIND == kKindTri ? kResolveWarps : 1][kResolveChunk];
	__shared__ uint32_t sOff[kResolveWarps][32];
	__shared__ uint32_t sSpan[kResolveWarps][32];
	/* the warp's tile of the depth and winner planes, moved by TMA */
	constexpr bool kTma = TMA && !MULTI && LATE_FS == 0;
	__shared__ __align__(128) ResolveTiles<kTma> tt;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t tile = blockIdx.x * kResolveWarps + warp;
	if (tile >= numTiles || P.ctr->abort) return;
	const uint32_t s = P.tileStart[tile], e = P.tileEnd[tile];
	if (s >= e) return;
	if (LATE_FS == 0 && e - s > P.heavyItems) return;  /* k_resolve_heavy's */
	const DrawState& st = P.st;
	const TileCtx c = tileCtx<MULTI>(P, tile);
	const int x0 = c.x0, y0 = c.y0;
	/* the depth tile's copy runs while the first chunk's coverage is found */
	bool tma = false, tmaStore = false;
	uint32_t mb = 0;
	if constexpr (kTma) {
		tma = (P.tma & kTmaResolveLoad) != 0;
		tmaStore = (P.tma & kTmaResolveStore) != 0;
		mb = smemAddr(&tt.bar[warp]);
		if (tma) {
			if (lane == 0) {
				mbarInit(mb, 1);
				fenceMbarInit();
				mbarArriveExpectTx(mb, 64 * 4);
				tmaLoad2d(smemAddr(tt.depth[warp]), &P.tmDepth, x0, y0, mb);
			}
			__syncwarp();
		}
	}
	bool depthIn = !tma;

	float depth[2];
	uint32_t sten[2], col[2];
	int32_t win[2];
	bool ok[2];
	size_t idx[2];
	int gx[2], gy[2];
#pragma unroll
	for (int p = 0; p < 2; ++p) {
		const int q = lane + 32 * p;
		gx[p] = x0 + (q & 7);
		gy[p] = y0 + (q >> 3);
		const bool valid = gx[p] < c.W && gy[p] < c.H;
		idx[p] = valid ? (size_t) gy[p] * c.W + gx[p] : 0;
		depth[p] = valid && !tma ? c.depth[idx[p]] : 0.0f;
		sten[p] = valid ? c.stencil[idx[p]] : 0u;
		col[p] = 0;
		win[p] = -1;
		/* line fragments were scissor-tested on their logical coordinates */
		ok[p] = valid && (KIND == kKindLineFrag || scissorPass(st, gx[p], gy[p]));
	}
	unsigned long long frags = 0;
	for (uint32_t b = s; b < e; b += kResolveChunk) {
		const uint32_t n = min((uint32_t) kResolveChunk, e - b);
		unsigned long long mask = 0;
		uint32_t item = 0, flags = 0;
		if (KIND == kKindTri) {
			/* triangles: coverage over flattened (item, row) pairs so that the
			 * lanes share the work whatever the items' sizes */
			uint32_t rows = 0, span = 0;
			if ((uint32_t) lane < n) {
				item = vals[b + lane];
				const TriRaster R = P.triR[item];
				sRec[warp][lane] = R;
				flags = R.flags;
				rows = triSpan(R, x0, y0, span);
			}
			uint32_t incl = rows;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
				if (lane >= o) incl += y;
			}
			const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
			sOff[warp][lane] = incl - rows;
			sSpan[warp][lane] = span;
			sMask[warp][lane] = 0;
			__syncwarp();
			for (uint32_t pr = lane; pr < total; pr += 32) {
				const int j = findOwner<32>(sOff[warp], pr);
				const uint32_t sp = sSpan[warp][j];
				const int xs = x0 + (int) (sp & 15u), xe = x0 + (int) ((sp >> 4) & 15u);
				const int y = y0 + (int) ((sp >> 8) & 15u) + (int) (pr - sOff[warp][j]);
				const unsigned long long bits = triRow(P, sRec[warp][j], x0, y0, xs, xe, y, sDep[warp][j]);
				if (bits) atomicOr(&sMask[warp][j], bits);
			}
			__syncwarp();
		} else {
			if ((uint32_t) lane < n) {
				item = vals[b + lane];
				coverage<KIND>(P, item, x0, y0, mask, sDep[warp][lane], flags);
			}
			sMask[warp][lane] = mask;
		}
		sItem[warp][lane] = item;
		sFlag[warp][lane] = flags;
		__syncwarp();
		if constexpr (kTma) {
			if (!depthIn) {
				/* bounded wait for the depth tile; on a timeout the error is
				 * recorded and the copy waited for once more before leaving */
				if (!mbarWait(mb, 0, P.spinLimit)) {
					if (lane == 0) atomicOr(&P.ctr->errors, kErrSpin);
					mbarWait(mb, 0, P.spinLimit);
					return;
				}
#pragma unroll
				for (int p = 0; p < 2; ++p) depth[p] = tt.depth[warp][lane + 32 * p];
				depthIn = true;
			}
		}
#pragma unroll
		for (int p = 0; p < 2; ++p) {
			if (!ok[p]) continue;
			const int q = lane + 32 * p;
			uint32_t m = 0;
			for (uint32_t j = 0; j < n; ++j) m |= (uint32_t) ((sMask[warp][j] >> q) & 1ull) << j;
			frags += __popc(m);
			while (m) {
				const int j = __ffs(m) - 1;
				m &= m - 1;
				const bool front = (sFlag[warp][j] & 1u) != 0;
				const StencilFace& sf = front ? st.front : st.back;
				float d = sDep[warp][j][q];
				if (st.stencilEnabled && !stencilCompare(sf.ref, sten[p], sf.mask, sf.func)) {
					sten[p] = stencilApply(sf.sfail, sten[p], sf.ref, sf.writeMask);
					continue;
				}
				if (LATE_FS == 0) {
					if (st.depthTest && !depthCompare(st.depthOp, d, depth[p])) {
						if (st.stencilEnabled) sten[p] = stencilApply(sf.dfail, sten[p], sf.ref, sf.writeMask);
						continue;
					}
				} else {
					SRPFragmentShaderOut out;
					shadeItem<KIND, LATE_FS>(P, c.uniform, c.primBase, sItem[warp][j], gx[p], gy[p], out);
					if (!isnan(out.fragDepth)) d = out.fragDepth;
					if (st.depthTest && !depthCompare(st.depthOp, d, depth[p])) {
						if (st.stencilEnabled) sten[p] = stencilApply(sf.dfail, sten[p], sf.ref, sf.writeMask);
						continue;
					}
					col[p] = packColor(out.color);
				}
				if (st.stencilEnabled) sten[p] = stencilApply(sf.pass, sten[p], sf.ref, sf.writeMask);
				win[p] = (int32_t) sItem[warp][j];
				if (st.depthTest && st.depthWrite) depth[p] = d;
			}
		}
		__syncwarp();
	}
	if (tmaStore) {
		/* depth and winner tiles back by TMA (the parts beyond the plane's
		 * edge are not written); the 8-byte stencil rows are below TMA's
		 * 16-byte row minimum and are stored directly */
		if constexpr (kTma) {
#pragma unroll
			for (int p = 0; p < 2; ++p) {
				tt.depth[warp][lane + 32 * p] = depth[p];
				tt.winner[warp][lane + 32 * p] = win[p];
				if (gx[p] < c.W && gy[p] < c.H) c.stencil[idx[p]] = (uint8_t) sten[p];
			}
			fenceProxyAsync();
			__syncwarp();
			if (lane == 0) {
				tmaStore2d(&P.tmDepth, x0, y0, smemAddr(tt.depth[warp]));
				tmaStore2d(&P.tmWinner, x0, y0, smemAddr(tt.winner[warp]));
				bulkCommit();
				bulkWaitRead();
			}
			__syncwarp();
		}
	} else {
#pragma unroll
		for (int p = 0; p < 2; ++p) {
			if (!(gx[p] < c.W && gy[p] < c.H)) continue;
			c.depth[idx[p]] = depth[p];
			c.stencil[idx[p]] = (uint8_t) sten[p];
			if (LATE_FS == 0) c.winner[idx[p]] = win[p];
			else if (win[p] >= 0) c.color[idx[p]] = col[p];
		}
	}
	if (KIND != kKindLineFrag) {
		for (int o = 16; o; o >>= 1) frags += __shfl_xor_sync(0xFFFFFFFFu, frags, o);
		if (lane == 0 && frags) atomicAdd(&P.ctr->fragments, frags);
	}
}

/* Applies one fragment to a pixel's depth/stencil state (early depth test;
 * src/raster/fragment.c:63-125). Returns true if it reached the colour write. */
__device__ __forceinline__ bool applyFragment(const DrawState& st, bool front, float d, float& depth, uint32_t& sten)
{
	const StencilFace& sf = front ? st.front : st.back;
	if (st.stencilEnabled && !stencilCompare(sf.ref, sten, sf.mask, sf.func)) {
		sten = stencilApply(sf.sfail, sten, sf.ref, sf.writeMask);
		return false;
	}
	if (st.depthTest && !depthCompare(st.depthOp, d, depth)) {
		if (st.stencilEnabled) sten = stencilApply(sf.dfail, sten, sf.ref, sf.writeMask);
		return false;
	}
	if (st.stencilEnabled) sten = stencilApply(sf.pass, sten, sf.ref, sf.writeMask);
	if (st.depthTest && st.depthWrite) depth = d;
	return true;
}

/* Light tiles of line fragments (early depth test). Every item is one
 * fragment on one pixel, so no coverage masks are needed: a warp takes 32
 * fragments at a time, the lanes whose fragments land on the same pixel find
 * each other with match.any, and the first of them applies the group's
 * fragments in item order to that pixel's depth/stencil state, which the
 * warp keeps in shared memory for the whole tile. */
__global__ void __launch_bounds__(kResolveWarps * 32) k_resolve_frags(const __grid_constant__ DrawParams P,
                                                                     const uint32_t* vals, uint32_t numTiles)
{
	gridDepSync();
	__shared__ float sDepth[kResolveWarps][64];
	__shared__ uint32_t sSten[kResolveWarps][64];
	__shared__ int32_t sWin[kResolveWarps][64];
	__shared__ float sFd[kResolveWarps][32];
	__shared__ uint32_t sFi[kResolveWarps][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t tile = blockIdx.x * kResolveWarps + warp;
	if (tile >= numTiles || P.ctr->abort) return;
	const uint32_t s = P.tileStart[tile], e = P.tileEnd[tile];
	if (s >= e || e - s > P.heavyItems) return;  /* empty, or k_resolve_heavy's */
	const DrawState& st = P.st;
	const TileCtx c = tileCtx<false>(P, tile);
	const int x0 = c.x0, y0 = c.y0;
	size_t idx[2];
	bool valid[2];
#pragma unroll
	for (int p = 0; p < 2; ++p) {
		const int q = lane + 32 * p;
		const int gx = x0 + (q & 7), gy = y0 + (q >> 3);
		valid[p] = gx < c.W && gy < c.H;
		idx[p] = valid[p] ? (size_t) gy * c.W + gx : 0;
		sDepth[warp][q] = valid[p] ? c.depth[idx[p]] : 0.0f;
		sSten[warp][q] = valid[p] ? c.stencil[idx[p]] : 0u;
		sWin[warp][q] = -1;
	}
	__syncwarp();
	for (uint32_t b = s; b < e; b += 32) {
		const uint32_t n = min(32u, e - b);
		int q = -1;
		float d = 0.0f;
		uint32_t item = 0;
		if ((uint32_t) lane < n) {
			item = vals[b + lane];
			const LineFrag F = P.frags[item];
			/* the logical pixel, as the reference indexes it (px may equal the width) */
			int gx, gy;
			lineFragPixel(st.W, F.px, F.py, gx, gy);
			const int qq = (gy - y0) * kTile + (gx - x0);
			if (qq >= 0 && qq < 64) q = qq;
			d = F.depth;
		}
		sFd[warp][lane] = d;
		sFi[warp][lane] = item;
		const unsigned peers = __match_any_sync(0xFFFFFFFFu, q);
		__syncwarp();
		if (q >= 0 && lane == __ffs(peers) - 1) {
			float depth = sDepth[warp][q];
			uint32_t sten = sSten[warp][q];
			int32_t win = sWin[warp][q];
			for (unsigned m = peers; m; m &= m - 1) {
				const int j = __ffs(m) - 1;
				if (applyFragment(st, true, sFd[warp][j], depth, sten)) win = (int32_t) sFi[warp][j];
			}
			sDepth[warp][q] = depth;
			sSten[warp][q] = sten;
			sWin[warp][q] = win;
		}
		__syncwarp();
	}
#pragma unroll
	for (int p = 0; p < 2; ++p) {
		if (!valid[p]) continue;
		const int q = lane + 32 * p;
		c.depth[idx[p]] = sDepth[warp][q];
		c.stencil[idx[p]] = (uint8_t) sSten[warp][q];
		c.winner[idx[p]] = sWin[warp][q];
	}
}

/* Tiles with many items (typically far-away meshes whose thousands of tiny
 * triangles land in a handful of tiles): a CTA takes 256 consecutive items
 * at a time, every thread evaluates one item's coverage and depths, warp
 * ballots transpose the coverage into per-pixel item masks, and 64 pixel
 * owners then apply just the covering fragments, in item order. Work per
 * chunk is parallel over items; per pixel only real fragments are walked.
 * Heavy tiles come from a list built by k_tile_classify and are pulled by a
 * fixed grid of CTAs. */
template <int KIND, bool MULTI = false>
__global__ void __launch_bounds__(kHeavyThreads) k_resolve_heavy(const __grid_constant__ DrawParams P,
                                                                const uint32_t* vals, const uint32_t* heavy)
{
	gridDepSync();
	extern __shared__ float hDep[];                 /* [kHeavyThreads][kDepRow] */
	__shared__ uint32_t ballots[kHeavyThreads / 32][64];
	__shared__ uint32_t hFlag[kHeavyThreads], hItem[kHeavyThreads];

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const DrawState& st = P.st;
	const uint32_t nHeavy = P.ctr->abort ? 0u : P.ctr->nonEmptyTiles;
	for (uint32_t h = blockIdx.x; h < nHeavy; h += gridDim.x) {
		const uint32_t tile = heavy[h];
		const uint32_t s = P.tileStart[tile], e = P.tileEnd[tile];
		const TileCtx c = tileCtx<MULTI>(P, tile);
		const int x0 = c.x0, y0 = c.y0;
		const int gx = x0 + (tid & 7), gy = y0 + ((tid >> 3) & 7);
		const bool owner = tid < 64;
		const bool valid = owner && gx < c.W && gy < c.H;
		const size_t idx = valid ? (size_t) gy * c.W + gx : 0;
		float depth = valid ? c.depth[idx] : 0.0f;
		uint32_t sten = valid ? c.stencil[idx] : 0u;
		int32_t win = -1;
		const bool ok = valid && (KIND == kKindLineFrag || scissorPass(st, gx, gy));
		unsigned long long frags = 0;
		uint32_t curItem = 0;
		typename RecOf<KIND>::T cur = {};
		if (s + tid < e) { curItem = vals[s + tid]; cur = loadRec<KIND>(P, curItem); }
		for (uint32_t b = s; b < e; b += kHeavyThreads) {
			const uint32_t n = min((uint32_t) kHeavyThreads, e - b);
			unsigned long long mask = 0;
			uint32_t item = 0, flags = 0;
			if ((uint32_t) tid < n) {
				item = curItem;
				coverageRec<KIND>(P, cur, x0, y0, mask, hDep + tid * kDepRow, flags);
			}
			/* prefetch the next chunk's item while this one is resolved */
			if (b + kHeavyThreads + tid < e) {
				curItem = vals[b + kHeavyThreads + tid];
				cur = loadRec<KIND>(P, curItem);
			}
			hFlag[tid] = flags;
			hItem[tid] = item;
			uint32_t lo = 0, hi = 0;
#pragma unroll
			for (int q = 0; q < 64; ++q) {
				const uint32_t bq = __ballot_sync(0xFFFFFFFFu, (mask >> q) & 1ull);
				if (lane == (q & 31)) { if (q < 32) lo = bq; else hi = bq; }
			}
			ballots[warp][lane] = lo;
			ballots[warp][32 + lane] = hi;
			__syncthreads();
			if (ok) {
				const int q = tid;
				for (int w = 0; w < kHeavyThreads / 32; ++w) {
					uint32_t m = ballots[w][q];
					frags += __popc(m);
					while (m) {
						const int j = w * 32 + __ffs(m) - 1;
						m &= m - 1;
						if (applyFragment(st, (hFlag[j] & 1u) != 0, hDep[j * kDepRow + q], depth, sten))
							win = (int32_t) hItem[j];
					}
				}
			}
			__syncthreads();
		}
		if (valid) {
			c.depth[idx] = depth;
			c.stencil[idx] = (uint8_t) sten;
			c.winner[idx] = win;
		}
		if (KIND != kKindLineFrag && warp < 2) {
			for (int o = 16; o; o >>= 1) frags += __shfl_xor_sync(0xFFFFFFFFu, frags, o);
			if (lane == 0 && frags) atomicAdd(&P.ctr->fragments, frags);
		}
	}
}

/* Lists the tiles with more than P.heavyItems items for k_resolve_heavy. */
__global__ void k_tile_classify(const __grid_constant__ DrawParams P, uint32_t numTiles, uint32_t* heavy)
{
	gridDepSync();
	const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= numTiles || P.ctr->abort) return;
	const uint32_t n = P.tileEnd[t] - P.tileStart[t];
	if (P.tileEnd[t] > P.tileStart[t] && n > P.heavyItems) heavy[atomicAdd(&P.ctr->nonEmptyTiles, 1u)] = t;
}

/* ------------------------------------------------------------ launchers */

static unsigned tileBlocks(uint32_t numTiles) { return (numTiles + kResolveWarps - 1) / kResolveWarps; }

template <int KIND, bool MULTI = false>
static void launchHeavy(const DrawParams& P, const uint32_t* vals, uint32_t* heavy, cudaStream_t s)
{
	const int smem = kHeavyThreads * kDepRow * 4;
	cudaFuncSetAttribute(k_resolve_heavy<KIND, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
	const unsigned perSM = P.heavyCtasPerSM >= 1 && P.heavyCtasPerSM <= 3 ? P.heavyCtasPerSM : 3u;
	pdlLaunch(k_resolve_heavy<KIND, MULTI>, 152 * perSM, kHeavyThreads, smem, s, P, vals, heavy);
}

void launchResolve(const DrawParams& P, int kind, const uint32_t* vals, uint32_t numTiles, uint32_t* heavy, cudaStream_t s,
                   cudaStream_t aux, cudaEvent_t fork, cudaEvent_t join)
{
	const unsigned b = tileBlocks(numTiles);
	pdlLaunch(k_tile_classify, (numTiles + 255) / 256, 256, 0, s, P, numTiles, heavy);
	const bool split = aux && fork && join;
	cudaStream_t hs = s;
	if (split) {
		cudaEventRecord(fork, s);
		cudaStreamWaitEvent(aux, fork, 0);
		hs = aux;
	}
	const bool tma = (P.tma & (kTmaResolveLoad | kTmaResolveStore)) != 0;
	if (kind == kKindTri) {
		launchHeavy<kKindTri>(P, vals, heavy, hs);
		if (tma) pdlLaunch(k_resolve<kKindTri, 0, false, true>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
		else pdlLaunch(k_resolve<kKindTri, 0>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	} else if (kind == kKindPoint) {
		launchHeavy<kKindPoint>(P, vals, heavy, hs);
		if (tma) pdlLaunch(k_resolve<kKindPoint, 0, false, true>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
		else pdlLaunch(k_resolve<kKindPoint, 0>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	} else {
		launchHeavy<kKindLineFrag>(P, vals, heavy, hs);
		pdlLaunch(k_resolve_frags, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	}
	if (split) {
		cudaEventRecord(join, aux);
		cudaStreamWaitEvent(s, join, 0);
	}
}

bool shadeSupportsLateDepth(int fsId) { return fsId == SRP_GPU_FS_DEPTH_OVERWRITE; }

void launchResolveLate(const DrawParams& P, int kind, const uint32_t* vals, uint32_t numTiles, cudaStream_t s)
{
	const unsigned b = tileBlocks(numTiles);
	if (kind == kKindTri) pdlLaunch(k_resolve<kKindTri, SRP_GPU_FS_DEPTH_OVERWRITE>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	else if (kind == kKindPoint) pdlLaunch(k_resolve<kKindPoint, SRP_GPU_FS_DEPTH_OVERWRITE>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	else pdlLaunch(k_resolve<kKindLineFrag, SRP_GPU_FS_DEPTH_OVERWRITE>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
}

void launchResolveMulti(const DrawParams& P, const uint32_t* vals, uint32_t numTiles, uint32_t* heavy, cudaStream_t s,
                        cudaStream_t aux, cudaEvent_t fork, cudaEvent_t join)
{
	const unsigned b = tileBlocks(numTiles);
	pdlLaunch(k_tile_classify, (numTiles + 255) / 256, 256, 0, s, P, numTiles, heavy);
	const bool split = aux && fork && join;
	cudaStream_t hs = s;
	if (split) {
		cudaEventRecord(fork, s);
		cudaStreamWaitEvent(aux, fork, 0);
		hs = aux;
	}
	launchHeavy<kKindTri, true>(P, vals, heavy, hs);
	pdlLaunch(k_resolve<kKindTri, 0, true>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	if (split) {
		cudaEventRecord(join, aux);
		cudaStreamWaitEvent(s, join, 0);
	}
}


}  // namespace srpg
