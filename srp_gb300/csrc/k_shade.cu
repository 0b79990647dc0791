/* Deferred shading and learned shading of the per-tile pipeline (the
 * resolve is in k_raster.cu): the winning fragment of each pixel is shaded
 * once, by the program's fragment shader (k_shade) or by the learned network
 * on the tensor cores with its judge (k_shade_learned5, k_judge_learned).
 * Shading only colours the pixel; coverage, depth and stencil are final
 * before it runs. So this unit is built with floating-point contraction
 * allowed: the colour is held to 1/255 per channel, not to the bit. */
#include <cuda_runtime.h>
#include <stdint.h>

#include "raster_common.cuh"
#include "launch.cuh"
#include "mlp.h"
#include "tc5.cuh"
#include "tma.cuh"

namespace srpg {
/* The colour of the winning fragment at pixel (gx, gy): the shader run on the
 * item, and for the shader that learned shading stands in for, a training
 * sample on the pixels the capture picks. */
template <int KIND, int FS>
__device__ __forceinline__ void shadeWinner(const DrawParams& P, const TileCtx& c, int32_t w, int gx, int gy,
                                            SRPFragmentShaderOut& out)
{
	if constexpr (KIND == kKindTri && FS == SRP_GPU_FS_MARBLE) {
		uint32_t words[kMaxVaryingWords];
		SRPFragmentShaderIn in;
		fragmentIn<KIND>(P, c.uniform, c.primBase, (uint32_t) w, gx, gy, in, words);
		runShader<FS>(in, out);
		if (P.capture && pixelSampled(gx, gy, P.sampleSeed + c.d, P.captureEvery))
			captureSample(P, c.uniform, words, out);
	} else {
		shadeItem<KIND, FS>(P, c.uniform, c.primBase, (uint32_t) w, gx, gy, out);
	}
}

/* The TMA variant of deferred shading for the tile at (c.x0, c.y0), run by
 * its 64 threads (named barrier BAR): the tile's colour comes in by TMA
 * while the shaders run, the shaded pixels are written into it, and it goes
 * back whole by TMA (parts beyond the plane's edge are not written). */
template <int KIND, int FS, int BAR>
__device__ __forceinline__ void shadeTileTma(const DrawParams& P, const TileCtx& c, int q, uint32_t* sCol,
                                             unsigned long long* sBar)
{
	const uint32_t mb = smemAddr(sBar);
	if (q == 0) {
		mbarInit(mb, 1);
		fenceMbarInit();
		mbarArriveExpectTx(mb, 64 * 4);
		tmaLoad2d(smemAddr(sCol), &P.tmColor, c.x0, c.y0, mb);
	}
	asm volatile("bar.sync %0, 64;" ::"n"(BAR) : "memory");
	const int gx = c.x0 + (q & 7), gy = c.y0 + (q >> 3);
	const int32_t w = (gx < c.W && gy < c.H) ? c.winner[(size_t) gy * c.W + gx] : -1;
	uint32_t packed = 0;
	if (w >= 0) {
		SRPFragmentShaderOut out;
		shadeWinner<KIND, FS>(P, c, w, gx, gy, out);
		packed = packColor(out.color);
	}
	/* bounded wait; on a timeout the copy is waited for once more and the
	 * tile is left as it was */
	const bool got = mbarWait(mb, 0, P.spinLimit);
	uint32_t all;
	asm volatile(
	    "{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\tbar.red.and.pred b, %2, 64, a;\n\t"
	    "selp.u32 %0, 1, 0, b;\n\t}\n"
	    : "=r"(all)
	    : "r"((uint32_t) got), "n"(BAR)
	    : "memory");
	if (!all) {
		if (q == 0) atomicOr(&P.ctr->errors, kErrSpin);
		mbarWait(mb, 0, P.spinLimit);
		return;
	}
	if (w >= 0) sCol[q] = packed;
	fenceProxyAsync();
	asm volatile("bar.sync %0, 64;" ::"n"(BAR) : "memory");
	if (q == 0) {
		tmaStore2d(&P.tmColor, c.x0, c.y0, smemAddr(sCol));
		bulkCommit();
		bulkWaitRead();
	}
}

template <bool TMA> struct ShadeTiles {
	__align__(128) uint32_t color[kShadeTiles][64];
	unsigned long long bar[kShadeTiles];
};
template <> struct ShadeTiles<false> {};

/* Deferred shading: one shader invocation per pixel whose colour was written
 * by the resolve pass. TMA: the variant whose tiles move by TMA. */
template <int KIND, int FS, bool MULTI = false, bool TMA = false>
__global__ void __launch_bounds__(kShadeTiles * 64) k_shade(const __grid_constant__ DrawParams P, uint32_t numTiles)
{
	gridDepSync();
	/* one pixel a thread, two warps a tile */
	constexpr bool kTma = TMA && !MULTI;
	__shared__ __align__(128) ShadeTiles<kTma> st;
	const int t = threadIdx.x >> 6;
	const uint32_t tile = blockIdx.x * kShadeTiles + (uint32_t) t;
	const int q = threadIdx.x & 63;
	if (tile >= numTiles || P.ctr->abort) return;
	if (P.tileStart[tile] >= P.tileEnd[tile]) return;
	const TileCtx c = tileCtx<MULTI>(P, tile);
	if (MULTI && P.redo && !P.redo[c.d]) return;
	if constexpr (kTma) {
		static_assert(kShadeTiles == 2, "one named barrier per tile of the block");
		if (t == 0) shadeTileTma<KIND, FS, 1>(P, c, q, st.color[0], &st.bar[0]);
		else shadeTileTma<KIND, FS, 2>(P, c, q, st.color[1], &st.bar[1]);
		return;
	}
	const int x0 = c.x0, y0 = c.y0;
	{
		const int gx = x0 + (q & 7), gy = y0 + (q >> 3);
		if (gx >= c.W || gy >= c.H) return;
		const size_t idx = (size_t) gy * c.W + gx;
		const int32_t w = c.winner[idx];
		if (w < 0) return;
		SRPFragmentShaderOut out;
		shadeWinner<KIND, FS>(P, c, w, gx, gy, out);
		c.color[idx] = packColor(out.color);
	}
}

/* Learned shading on tcgen05. A CTA holds kLearnGroups independent groups of
 * 4 warps that share one copy of the weights in shared memory; each group
 * shades a pair of tiles (128 pixels, one per thread) at a time as one
 * 128-row MMA tile, with its own A tile, 64 TMEM columns, mbarrier and named
 * barrier, so that one group's fragment loads and encoding overlap another
 * group's MMA chain. Groups take the tile pairs in order from a counter of
 * the draw, one at a time, so that the CTAs end together. In a group each thread builds its pixel's encoded inputs
 * as row `gt` of the A tile; one thread issues each layer's MMAs into a
 * 128 x 64 fp32 accumulator in tensor memory; each warp reads its 32 lanes
 * (rows) back, adds the bias, applies ReLU and writes the next A tile, and
 * finally its pixels' colours. The judge runs afterwards as its own pass
 * (k_judge_learned). Every wait is bounded; on a timeout the group records
 * kErrSpin and stops, and the CTA releases its tensor memory and returns. */
constexpr int kLearnGroups = 6;
constexpr int kLearnThreads = 128 * kLearnGroups;
constexpr uint32_t kLearnCols = 512;   /* kLearnGroups x 64 columns, rounded up to a power of two */
constexpr size_t kLearnSmem = kTcWBytes + (size_t) kLearnGroups * kTcABytes + 208 * 4 + kLearnGroups * 8 + 16 +
                              kLearnGroups * 4;
static_assert(kLearnGroups * 64 <= (int) kLearnCols && kLearnCols <= 512, "TMEM columns");
static_assert(kLearnSmem <= 227 * 1024, "shared memory");

template <int KIND, bool MULTI>
__global__ void __launch_bounds__(kLearnThreads, 1) k_shade_learned5(const __grid_constant__ DrawParams P, uint32_t numTiles)
{
	gridDepSync();
	extern __shared__ __align__(1024) uint8_t tsm[];
	const int tid = threadIdx.x, warp = tid >> 5;
	const int g = warp >> 2, gt = tid & 127;          /* group, thread within the group */
	const uint32_t bar = 1u + (uint32_t) g;            /* the group's named barrier (0 is __syncthreads) */
	uint8_t* sW = tsm;
	uint8_t* sA = tsm + kTcWBytes + (size_t) g * kTcABytes;
	float* sB = (float*) (tsm + kTcWBytes + (size_t) kLearnGroups * kTcABytes);
	uint64_t* mbars = (uint64_t*) (sB + 208);
	uint32_t* tslot = (uint32_t*) (mbars + kLearnGroups);
	uint32_t* sNext = tslot + 4;                       /* per group: the pair it takes next */
	for (int i = tid; i < (int) (kTcWBytes / 16); i += kLearnThreads) ((uint4*) sW)[i] = ((const uint4*) P.mlpW5)[i];
	for (int i = tid; i < 3 * kMlpHid + kMlpOut; i += kLearnThreads) sB[i] = P.mlpB[i];
	const uint32_t mb = smemAddr(mbars + g);
	if (gt == 0) {
		mbarInit(mb, 1);
		sNext[g] = atomicAdd(&P.ctr->learnedPairs, 1u);
	}
	if (warp == 0) tcAlloc(smemAddr(tslot), kLearnCols);
	fenceProxyAsync();
	tcFenceBefore();
	__syncthreads();
	tcFenceAfter();
	const uint32_t tmemAll = *tslot;
	const uint32_t tmem = tmemAll + (uint32_t) (g * 64);
	const uint32_t laneBase = tmem + ((uint32_t) ((warp & 3) * 32) << 16);
	const uint32_t aAddr = smemAddr(sA), wAddr = smemAddr(sW);
	const int half = gt >> 6, q = gt & 63;
	uint32_t phase = 0;
	bool ok = P.ctr->abort == 0;
	const uint32_t pairs = (numTiles + 1) / 2;
	for (uint32_t pr = sNext[g]; ok && pr < pairs; pr = sNext[g]) {
		/* sNext[g] is rewritten only after the group's next barrier, once every thread has read it */
		const uint32_t tile = 2 * pr + (uint32_t) half;
		const bool have = tile < numTiles && P.tileStart[tile] < P.tileEnd[tile];
		TileCtx c = {};
		size_t idx = 0;
		int32_t win = -1;
		float x9[9] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
		if (have) {
			c = tileCtx<MULTI>(P, tile);
			const int gx = c.x0 + (q & 7), gy = c.y0 + (q >> 3);
			if (gx < c.W && gy < c.H) {
				idx = (size_t) gy * c.W + gx;
				win = c.winner[idx];
			}
			if (win >= 0) {
				uint32_t words[kMaxVaryingWords];
				SRPFragmentShaderIn in;
				fragmentIn<KIND>(P, c.uniform, c.primBase, (uint32_t) win, gx, gy, in, words);
				learnedInputs(c.uniform, words, x9);
			}
		}
		const bool any = namedSyncOr(bar, 128, win >= 0);
		uint32_t next = 0;
		if (gt == 0) next = atomicAdd(&P.ctr->learnedPairs, 1u);
		if (!any) {
			if (gt == 0) sNext[g] = next;
			namedSync(bar, 128);
			continue;
		}
#pragma unroll
		for (int f = 0; f < kMlpInPad; f += 2) {
			uint32_t v = 0;
			if (f < kMlpIn) {
				float sn, cs;
				__sincosf(mlpBandScale((f % 12) / 2) * x9[f / 12], &sn, &cs);
				v = packBf16(sn, cs);
			}
			*(uint32_t*) (sA + tcOffset(gt, f, kMlpInPad)) = v;
		}
		fenceProxyAsync();
		tcFenceBefore();
		namedSync(bar, 128);
		float rgb[3] = { 0.f, 0.f, 0.f };
		for (int layer = 0; layer < 4; ++layer) {
			/* a failure-detection test issues nothing for layer 1: its wait
			 * runs out with no MMA in flight */
			if (gt == 0 && !(layer == 1 && (P.waitTest & kWaitTestLearned))) {
				tcFenceAfter();
				const int K = layer == 0 ? kMlpInPad : 64;
				const uint32_t w = wAddr + (layer == 0 ? kTcW1 : layer == 1 ? kTcW2 : layer == 2 ? kTcW3 : kTcW4);
				tcLayer(tmem, aAddr, w, K, layer < 3 ? 64 : 16);
				tcCommit(mb);
				/* the counter's answer is awaited here, beside the first layer's MMAs */
				if (layer == 0) sNext[g] = next;
			}
			const bool got = mbarWait(mb, phase, P.spinLimit);
			phase ^= 1u;
			if (!namedSyncAnd(bar, 128, got)) { ok = false; break; }
			tcFenceAfter();
			if (layer < 3) {
				const float* bias = sB + 64 * layer;
				for (int col = 0; col < 64; col += 16) {
					float v[16];
					tcLoad16(laneBase + (uint32_t) col, v);
#pragma unroll
					for (int i = 0; i < 16; i += 2) {
						const float x0 = fmaxf(v[i] + bias[col + i], 0.0f), x1 = fmaxf(v[i + 1] + bias[col + i + 1], 0.0f);
						*(uint32_t*) (sA + tcOffset(gt, col + i, 64)) = packBf16(x0, x1);
					}
				}
				fenceProxyAsync();
			} else {
				float v[16];
				tcLoad16(laneBase, v);
				for (int k = 0; k < 3; ++k) rgb[k] = clamp01f(v[k] + sB[3 * kMlpHid + k]);
			}
			tcFenceBefore();
			namedSync(bar, 128);
		}
		if (!ok) break;
		if (win >= 0) {
			const float col[4] = { rgb[0], rgb[1], rgb[2], 1.0f };
			c.color[idx] = packColor(col);
		}
	}
	if (!ok && P.ctr->abort == 0 && gt == 0) atomicOr(&P.ctr->errors, kErrSpin);
	tcFenceBefore();
	__syncthreads();
	tcFenceAfter();
	if (warp == 0) tcDealloc(tmemAll, kLearnCols);
}

/* The judge of learned shading, a pass of its own after k_shade_learned5:
 * 1 pixel in judgeEvery is shaded again by the plain shader (FS), and per
 * draw the squared difference between the network's stored colour and the
 * shader's (both as the 8-bit channels the framebuffer holds, in [0, 1]
 * units) and the largest channel difference are accumulated. Run at the
 * deferred-shading pass's occupancy, so that the few judged pixels do not
 * hold up the tensor-core kernel's tile pairs. */
template <int KIND, int FS, bool MULTI>
__global__ void __launch_bounds__(kShadeTiles * 64) k_judge_learned(const __grid_constant__ DrawParams P, uint32_t numTiles)
{
	gridDepSync();
	const uint32_t tile = blockIdx.x * kShadeTiles + (threadIdx.x >> 6);
	const int q = threadIdx.x & 63;
	/* tile-level exits are uniform over each warp: a warp's 32 pixels lie in one tile */
	if (tile >= numTiles || P.ctr->abort) return;
	if (P.tileStart[tile] >= P.tileEnd[tile]) return;
	const TileCtx c = tileCtx<MULTI>(P, tile);
	const int gx = c.x0 + (q & 7), gy = c.y0 + (q >> 3);
	double err = 0.0, chans = 0.0;
	float worst = 0.0f;
	if (gx < c.W && gy < c.H && pixelSampled(gx, gy, P.sampleSeed + c.d, P.judgeEvery)) {
		const size_t idx = (size_t) gy * c.W + gx;
		const int32_t w = c.winner[idx];
		if (w >= 0) {
			SRPFragmentShaderOut ref;
			shadeItem<KIND, FS>(P, c.uniform, c.primBase, (uint32_t) w, gx, gy, ref);
			const uint32_t net = c.color[idx], plain = packColor(ref.color);
			for (int k = 0; k < 3; ++k) {
				const int sh = 24 - 8 * k;
				const float dlt = (float) ((int) ((net >> sh) & 0xFFu) - (int) ((plain >> sh) & 0xFFu)) / 255.0f;
				err += (double) dlt * dlt;
				worst = fmaxf(worst, fabsf(dlt));
			}
			chans = 3.0;
		}
	}
	for (int o = 16; o; o >>= 1) {
		err += __shfl_xor_sync(0xFFFFFFFFu, err, o);
		chans += __shfl_xor_sync(0xFFFFFFFFu, chans, o);
		worst = fmaxf(worst, __shfl_xor_sync(0xFFFFFFFFu, worst, o));
	}
	if ((threadIdx.x & 31) == 0 && chans > 0.0) {
		atomicAdd(&P.judge[2 * c.d], err);
		atomicAdd(&P.judge[2 * c.d + 1], chans);
		atomicMax(&P.judgeMax[c.d], __float_as_uint(worst));
	}
}

/* ------------------------------------------------------------ launchers */

template <int KIND, bool MULTI = false, bool TMA = false>
static void shadeKind(const DrawParams& P, uint32_t numTiles, cudaStream_t s)
{
	const unsigned b = (numTiles + kShadeTiles - 1) / kShadeTiles;
	const unsigned t = kShadeTiles * 64;
	switch (P.fsId) {
	case SRP_GPU_FS_VARYING_COLOR: pdlLaunch(k_shade<KIND, SRP_GPU_FS_VARYING_COLOR, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_SOLID: pdlLaunch(k_shade<KIND, SRP_GPU_FS_SOLID, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_PRIMITIVE_ID: pdlLaunch(k_shade<KIND, SRP_GPU_FS_PRIMITIVE_ID, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_TEXTURE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_TEXTURE, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_TEXTURE_MODULATE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_TEXTURE_MODULATE, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_BLINN_PHONG: pdlLaunch(k_shade<KIND, SRP_GPU_FS_BLINN_PHONG, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_MARBLE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_MARBLE, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_DEPTH_OVERWRITE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_DEPTH_OVERWRITE, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_FRAGCOORD: pdlLaunch(k_shade<KIND, SRP_GPU_FS_FRAGCOORD, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_FLAT_INT: pdlLaunch(k_shade<KIND, SRP_GPU_FS_FLAT_INT, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_MIXED: pdlLaunch(k_shade<KIND, SRP_GPU_FS_MIXED, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_BYTE_PALETTE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_BYTE_PALETTE, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_PRIMITIVE_MOD: pdlLaunch(k_shade<KIND, SRP_GPU_FS_PRIMITIVE_MOD, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_TEXTURE_LOD: pdlLaunch(k_shade<KIND, SRP_GPU_FS_TEXTURE_LOD, MULTI, TMA>, b, t, 0, s, P, numTiles); break;
	case kFsLearned:
		if constexpr (KIND == kKindTri) {
			/* one CTA per SM, its groups looping over the tile pairs */
			const unsigned pairs = (numTiles + 1) / 2;
			const unsigned need = (pairs + kLearnGroups - 1) / kLearnGroups;
			const unsigned blocks = need < 152u ? (need ? need : 1u) : 152u;
			cudaFuncSetAttribute(k_shade_learned5<KIND, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kLearnSmem);
			pdlLaunch(k_shade_learned5<KIND, MULTI>, blocks, kLearnThreads, kLearnSmem, s, P, numTiles);
			pdlLaunch(k_judge_learned<KIND, SRP_GPU_FS_MARBLE, MULTI>, b, t, 0, s, P, numTiles);
		}
		break;
	default: break;
	}
}

void launchShade(const DrawParams& P, int kind, uint32_t numTiles, cudaStream_t s)
{
	if (P.tma & kTmaShade) {
		if (kind == kKindTri) shadeKind<kKindTri, false, true>(P, numTiles, s);
		else if (kind == kKindPoint) shadeKind<kKindPoint, false, true>(P, numTiles, s);
		else shadeKind<kKindLineFrag, false, true>(P, numTiles, s);
		return;
	}
	if (kind == kKindTri) shadeKind<kKindTri>(P, numTiles, s);
	else if (kind == kKindPoint) shadeKind<kKindPoint>(P, numTiles, s);
	else shadeKind<kKindLineFrag>(P, numTiles, s);
}

void launchShadeMulti(const DrawParams& P, uint32_t numTiles, cudaStream_t s) { shadeKind<kKindTri, true>(P, numTiles, s); }

}  // namespace srpg
