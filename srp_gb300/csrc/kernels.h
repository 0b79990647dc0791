/* Draw parameters passed to every kernel (as a __grid_constant__ parameter,
 * so the user uniform inside it is read straight from the constant bank) and
 * the host-side launch wrappers of each kernel translation unit. */
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include "gpu_types.h"

namespace srpg {

struct DrawParams {
	DrawState st;
	VaryingLayout L;
	int vsId, fsId;
	int prim;                      /* SRPPrimitive of the draw */
	int indexSize;                 /* 0: non-indexed, else 1/2/4/8 bytes */
	int shadeAll;                  /* indexed: shade every vertex of the buffer instead of
	                                  the index range found by k_index_range */
	const void* indices;           /* device copy of the index buffer */
	unsigned long long start, count;
	const unsigned char* vertices; /* device copy of the vertex buffer (user AoS) */
	unsigned long long nVertices;
	int stride;                    /* bytes per vertex */
	int nIn;                       /* input primitives of this draw */
	/* post-VS vertices: rows [0, nVertices) from the vertex shader, rows
	 * [clipBase, clipBase + clipCap) created by clipping */
	float4* clip;
	float4* vset0;                 /* per vertex: ndc x, ndc y, screen x, screen y */
	float4* vset1;                 /* per vertex inside the frustum: z_ndc/w, 1/w, z_ndc, 0 */
	uint8_t* codes;                /* per vertex: outcode bits (one byte, so that the
	                                  clip and cull tests of setup read 32 vertices a sector) */
	uint32_t* vary;
	uint32_t clipBase, clipCap;
	unsigned long long* minmax;    /* [0] min, [1] max vertex index referenced */
	/* primitives in submission order */
	TriRaster* triR;
	TriAttr* triA;
	LineRec* lines;
	PointRec* points;
	LineFrag* frags;               /* line draws: kRunFrags records per pair slot */
	uint32_t primCap;
	unsigned long long fragCap;    /* records in frags */
	/* line draws, after the sort: the sorted runs' block sums
	 * [runSumWords], and the record numbers of the fragments in sorted order
	 * [fragCap] */
	uint32_t* runSums;
	uint32_t* fragVals;
	/* (tile, item) pairs */
	uint32_t* keys;
	uint32_t* vals;
	uint32_t entryCap;
	/* triangles that need clipping: the pre-pass stores their polygon
	 * (count + vertex rows) and, per input triangle, its polygon slot */
	uint32_t* clipSlot;            /* [nIn], written only for clipped triangles */
	uint32_t* clipPolys;           /* [clipPolyCap][1 + kMaxPoly] */
	uint32_t clipPolyCap;
	/* filled triangles: each clipped triangle's fan, set up by the clip
	 * pre-pass, [clipPolyCap]: (triangles, pairs), and its triangles'
	 * records, [clipPolyCap][kClipFan] (TriAttr.pad = the triangle's pairs) */
	uint2* clipFan;
	TriRaster* clipR;
	TriAttr* clipA;
	uint4* bigJobs;                /* primitives covering many tiles */
	uint32_t bigCap;
	/* exact barycentrics of big triangles at every (row, tile column) start:
	 * rows x columns x 3 floats per triangle */
	float* table;
	unsigned long long tableCap;
	unsigned long long* lookback;  /* decoupled look-back status, one per block */
	/* framebuffer planes */
	uint32_t* color;
	float* depth;
	uint8_t* stencil;
	int32_t* winner;               /* last item that reached the colour write */
	uint32_t* tileStart;
	uint32_t* tileEnd;
	DeviceCounters* ctr;
	/* multi-draw pass (nDraws > 0, triangles in fill mode only): the draws'
	 * descriptors and prefix sums over the draws ([nDraws + 1] each) of input
	 * primitives, vertex rows, tiles and vertex-kernel blocks. primPrefix
	 * (surviving primitives before each draw) is written by k_setup_multi.
	 * Primitive, entry and tile numbers are then global over the pass. */
	const DrawDesc* draws;
	uint32_t nDraws;
	/* resolve tuning: tiles with more than heavyItems items are resolved by
	 * a CTA (k_resolve_heavy, heavyCtasPerSM CTAs per SM), the others by a
	 * warp (k_resolve) */
	uint32_t heavyItems, heavyCtasPerSM;
	const uint32_t* inPrefix;
	const uint32_t* vPrefix;
	const uint32_t* tPrefix;
	const uint32_t* blkPrefix;
	uint32_t* primPrefix;
	/* learned shading (fsId == kFsLearned): the MLP's bf16 weights and fp32
	 * biases; the plain shader that judges it (judgeFs) on 1 pixel in
	 * judgeEvery; per draw d (0 for a single draw) the judge's squared-error
	 * sum and channel count (judge[2d], judge[2d + 1]) and largest channel
	 * error (judgeMax[d], float bits). redo: a multi-draw shade pass that
	 * shades only the draws flagged there (fallback to the plain shader). */
	const void* mlpW5;            /* bf16 weights in the tcgen05 operand layout */
	const float* mlpB;
	int judgeFs;
	uint32_t judgeEvery, sampleSeed;
	double* judge;
	unsigned int* judgeMax;
	const uint8_t* redo;
	/* fragment capture for training: 1 pixel in captureEvery shaded by the
	 * plain shader adds (position, normal, view direction, colour) */
	float* capture;
	unsigned long long* captureCount;
	uint32_t captureCap, captureEvery;
	/* bounded device waits: polls before a wait gives up (0: the default),
	 * and the kWaitTest* signals withheld so that a wait runs out (tests of
	 * failure detection only) */
	uint32_t spinLimit, waitTest;
	/* tile copies by TMA (a single draw into a framebuffer whose width is a
	 * multiple of 4; tma = 0 otherwise): tensor maps of the depth, winner and
	 * colour planes, in 8 x 8 boxes of 32-bit pixels. kTmaResolveLoad: the
	 * light-tile resolve loads its depth tile through them; kTmaResolveStore:
	 * it stores its depth and winner tiles; kTmaShade: the deferred shading
	 * loads, updates and stores its colour tile. */
	uint32_t tma;
	alignas(64) CUtensorMap tmDepth;
	alignas(64) CUtensorMap tmWinner;
	alignas(64) CUtensorMap tmColor;
	alignas(16) unsigned char uniform[kMaxUniformBytes];
};

/* Parts of a draw whose framebuffer tiles move by TMA (DrawParams::tma). */
constexpr uint32_t kTmaResolveLoad = 1u, kTmaResolveStore = 2u, kTmaShade = 4u;

/* Signals a test can withhold (srpGpuSetWaitTest). */
constexpr uint32_t kWaitTestSetup = 1u;    /* block 0 of the ordered setup never publishes its prefix */
constexpr uint32_t kWaitTestLearned = 2u;  /* learned shading issues no MMAs (and no commit) for layer 1 */

/* Fragment-shader id of learned shading (not a user shader). */
constexpr int kFsLearned = 100;

constexpr int kTile = 8;              /* tile edge in pixels */
/* Ordered setup: blocks of 128 threads, at least 10 resident per SM (48
 * registers a thread). The block waits at its scan barriers for the
 * look-back, so more, smaller resident blocks keep the SM busy meanwhile. */
constexpr int kSetupThreads = 128;
constexpr int kSetupBlocksPerSM = 10;
constexpr int kSmallEntries = 16;     /* tiles a primitive may write inline */

/* k_front.cu */
void launchReset(const DrawParams& P, cudaStream_t s);
void launchIndexRange(const DrawParams& P, cudaStream_t s);
void launchVertex(const DrawParams& P, unsigned long long first, unsigned long long n, cudaStream_t s);
void launchSetup(const DrawParams& P, cudaStream_t s);
/* After setup: sets the abort flag when any count exceeds its buffer (or an
 * index was bad). Every later kernel reads its sizes from the counters, not
 * from the host, and does nothing once the flag is set, so a draw can be
 * enqueued to the end before the host has seen its counts. */
void launchCheck(const DrawParams& P, cudaStream_t s);
void launchClipPrepass(const DrawParams& P, cudaStream_t s);
/* jobsHint (the big-primitive count of a similar earlier draw) only sizes
 * the grids; the kernels loop over the count the device holds. */
void launchBigEntries(const DrawParams& P, uint32_t jobsHint, cudaStream_t s);
/* lambda tables of the big triangles (triangle draws) */
void launchLambdaTables(const DrawParams& P, uint32_t jobsHint, cudaStream_t s);
void launchLineFrags(const DrawParams& P, cudaStream_t s);
/* Line draws: turns the sorted runs back into fragments (fragVals, and the
 * tile ranges over them, in place of launchTileRanges). */
void launchRunExpand(const DrawParams& P, const uint32_t* keys, const uint32_t* vals, uint32_t numTiles, cudaStream_t s);
uint32_t runSumWords(uint32_t entryCap);
/* Largest pair capacity of a line draw (a run's slot shares its value word
 * with its fragment count). */
constexpr uint32_t kMaxLineEntries = (1u << kRunCountShift) - 1u;
/* k_front.cu, multi-draw pass */
void launchVertexMulti(const DrawParams& P, uint32_t blocks, int maxStride, cudaStream_t s);
void launchClipPrepassMulti(const DrawParams& P, cudaStream_t s);
void launchSetupMulti(const DrawParams& P, cudaStream_t s);
void launchBigEntriesMulti(const DrawParams& P, uint32_t jobsHint, cudaStream_t s);
void launchLambdaTablesMulti(const DrawParams& P, uint32_t jobsHint, cudaStream_t s);
/* k_bin.cu */
/* Sorts the draw's (tile, item) pairs by tile, stably; their number is read
 * from the counters (at most P.entryCap, the size the scratch is for). */
void sortEntries(const DrawParams& P, uint32_t keyBits, uint32_t* keysAlt, uint32_t* valsAlt,
                 uint32_t* hist, uint32_t* partials, uint32_t** keysOut, uint32_t** valsOut, cudaStream_t s);
void launchTileRanges(const DrawParams& P, const uint32_t* keys, uint32_t numTiles, cudaStream_t s);
size_t sortHistWords(uint32_t n);
size_t sortPartialWords(uint32_t n);
/* k_raster.cu */
/* Heavy tiles (k_resolve_heavy) and light tiles (k_resolve) are disjoint: with
 * an auxiliary stream and two events the heavy kernel runs on `aux` beside
 * the light one, joined back into `s` before the function's work ends;
 * without them both run on `s` in turn. */
void launchResolve(const DrawParams& P, int kind, const uint32_t* vals, uint32_t numTiles, uint32_t* heavy,
                   cudaStream_t s, cudaStream_t aux = nullptr, cudaEvent_t fork = nullptr,
                   cudaEvent_t join = nullptr);
void launchResolveMulti(const DrawParams& P, const uint32_t* vals, uint32_t numTiles, uint32_t* heavy, cudaStream_t s,
                        cudaStream_t aux, cudaEvent_t fork, cudaEvent_t join);
void launchShadeMulti(const DrawParams& P, uint32_t numTiles, cudaStream_t s);
/* k_raster.cu, deferred shading */
void launchShade(const DrawParams& P, int kind, uint32_t numTiles, cudaStream_t s);
bool shadeSupportsLateDepth(int fsId);
void launchResolveLate(const DrawParams& P, int kind, const uint32_t* vals, uint32_t numTiles, cudaStream_t s);

}  // namespace srpg
