/* srpGpuDrawFixedScratch: a draw that allocates nothing.
 *
 * The ordinary draws (srpDrawIndexBuffer, srpDrawVertexBuffer) keep their
 * scratch buffers in pools that grow with cudaMalloc, freeing the smaller
 * buffer, whenever a draw needs more than the draws before it. Some callers
 * cannot have that happen in the middle of a frame:
 *   - a renderer whose other CUDA streams must keep running: cudaFree waits
 *     for all work on the device, so one pool growth stalls every stream;
 *   - a program that has handed the rest of device memory to a caching
 *     allocator (PyTorch's, for one) or shares the GPU with other processes:
 *     an allocation made mid-frame can fail where the previous frame worked;
 *   - a service that admits work by a device-memory budget fixed up front.
 * This entry point runs the same kernels in the same order as the ordinary
 * draw, but carves every scratch buffer out of one array of fixed size that
 * is part of the library's device image (fixedScratch below). It calls no
 * cudaMalloc, cudaFree or other allocating routine. The array lives in this
 * translation unit, which has no kernels, so with lazy module loading (the
 * CUDA default) it takes device memory only in processes that call this
 * entry point.
 *
 * It has no counterpart in kitrofimov/srp; its draw semantics are those of
 * drawBuffer (src/pipeline/draw.c:63-82) like the ordinary draw's. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "srp/gpu.h"
#include "draw_internal.h"
#include "kernels.h"

using namespace srpg;

/* All fixed-scratch draws on a device share this array. */
static __device__ __align__(256) unsigned char fixedScratch[SRP_GPU_FIXED_SCRATCH_BYTES];

namespace {

constexpr const char* kFn = "srpGpuDrawFixedScratch";
constexpr int kMaxDevices = 64;
constexpr size_t kClipRows = 16384;          /* vertices created by clipping, per draw */
constexpr size_t kClipPolys = 4096;          /* triangles that need clipping, per draw */
constexpr size_t kMinBinBytes = 4u << 20;    /* left for tile entries and tables at least */

/* Device address of fixedScratch, per device ordinal; null until the first
 * call on that device has looked it up. */
unsigned char* scratchOnDevice[kMaxDevices];

DrawParams P;
DeviceCounters hostCounters;  /* pageable host copy of the draw's counters */

/* Set-up, once per device, with that device current: the address of the
 * array on the current device. Looking it up loads the library's device image
 * that holds it, which is why the first call on a device must not come
 * while a stream is being captured. */
unsigned char* scratchBase()
{
	int dev = -1;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
		fixedDrawError(kFn, "No usable CUDA device (%s)",
		               e != cudaSuccess ? cudaGetErrorString(e) : "device ordinal out of range");
		cudaGetLastError();
		return nullptr;
	}
	if (!scratchOnDevice[dev]) {
		void* p = nullptr;
		e = cudaGetSymbolAddress(&p, fixedScratch);
		if (e != cudaSuccess || !p) {
			fixedDrawError(kFn, "cudaGetSymbolAddress of the fixed scratch array failed on device %d: %s", dev,
			               cudaGetErrorString(e));
			cudaGetLastError();
			return nullptr;
		}
		scratchOnDevice[dev] = (unsigned char*) p;
	}
	return scratchOnDevice[dev];
}

/* Hands out 256-byte aligned offsets from the front of the array. */
struct Carver {
	size_t used = 0;
	size_t take(size_t bytes)
	{
		const size_t at = used;
		used += (bytes + 255) & ~(size_t) 255;
		return at;
	}
};

size_t round256(size_t b) { return (b + 255) & ~(size_t) 255; }

/* Scratch of the binning stage for E tile entries. */
size_t binBytes(size_t E, bool lineFrags)
{
	const size_t e = E ? E : 1;
	/* line draws: kRunFrags records and fragment numbers per pair slot, and
	 * the runs' block sums */
	const size_t lines = lineFrags ? round256(e * kRunFrags * sizeof(LineFrag)) + round256(e * kRunFrags * 4) +
	                                     round256((size_t) runSumWords((uint32_t) e) * 4)
	                               : 0;
	return 4 * round256(e * 4) + lines +
	       round256(sortHistWords((uint32_t) e) * 4) + round256(sortPartialWords((uint32_t) e) * 4 + 64);
}

bool launchedOk(const char* what)
{
	const cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) return true;
	fixedDrawError(kFn, "%s: %s", what, cudaGetErrorString(e));
	return false;
}

}  // namespace

extern "C" int srpGpuDrawFixedScratch(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                                      const SRPShaderProgram* sp, SRPPrimitive prim, size_t startIndex, size_t count)
{
	FixedDrawInfo info;
	const int prep = fixedDrawPrepare(P, ib, vb, fb, sp, prim, startIndex, count, info);
	if (prep != 0) return prep > 0 ? 0 : -1;
	unsigned char* base = scratchBase();
	if (!base) return -1;
	const cudaStream_t s = info.stream;

	/* parts whose size is known before anything runs */
	const size_t nV = (size_t) P.nVertices;
	const size_t rows = nV + kClipRows;
	const size_t nw = (size_t) std::max(P.L.nWords, 1);
	const size_t blocks = std::max<size_t>((info.nIn + kSetupThreads - 1) / kSetupThreads, 1);
	/* every input primitive once, plus the extra triangles of clipping: each
	 * of the kClipPolys clipped triangles fans out into up to kMaxPoly - 2 */
	const size_t primCap = std::min<size_t>((info.nIn + kClipPolys * (kMaxPoly - 3)) * info.outPer, 0x3FFFFFFFu);
	Carver cv;
	const size_t oCtr = cv.take(sizeof(DeviceCounters));
	const size_t oMinmax = cv.take(16);
	const size_t oLook = cv.take(blocks * 8);
	const size_t oClip = cv.take(rows * 16);
	const size_t oSet0 = cv.take(nV * 16 + 16);
	const size_t oSet1 = cv.take(nV * 16 + 16);
	const size_t oCodes = cv.take(nV + 16);
	const size_t oVary = cv.take(rows * nw * 4);
	const size_t oSlot = cv.take(info.nIn * 4 + 4);
	const size_t oPolys = cv.take(kClipPolys * (1 + kMaxPoly) * 4);
	size_t oPrimA = 0, oPrimB = 0, oFan = 0, oFanR = 0, oFanA = 0;
	if (info.kind == kKindTri) {
		oPrimA = cv.take(primCap * sizeof(TriRaster));
		oPrimB = cv.take(primCap * sizeof(TriAttr));
		oFan = cv.take(kClipPolys * sizeof(uint2));
		oFanR = cv.take(kClipPolys * kClipFan * sizeof(TriRaster));
		oFanA = cv.take(kClipPolys * kClipFan * sizeof(TriAttr));
	} else {
		oPrimA = cv.take(primCap * (info.kind == kKindPoint ? sizeof(PointRec) : sizeof(LineRec)));
	}
	const size_t bigCap = primCap;  /* room for every primitive, long-line queue included */
	const size_t oBig = cv.take(bigCap * 16);
	const size_t oStart = cv.take(((size_t) info.numTiles + 1) * 4);
	const size_t oEnd = cv.take(((size_t) info.numTiles + 1) * 4);
	const size_t oHeavy = cv.take(((size_t) info.numTiles + 1) * 4);
	const size_t oWinner = cv.take(info.pixels * 4 + 4);
	if (cv.used + kMinBinBytes > (size_t) SRP_GPU_FIXED_SCRATCH_BYTES) {
		fixedDrawError(kFn,
		               "Draw too large for the fixed scratch: %zu vertices, %zu primitives and a %zux%zu framebuffer "
		               "need %zu bytes before binning, and %zu more are kept for binning; the array holds %zu bytes",
		               nV, info.nIn * info.outPer, (size_t) P.st.W, (size_t) P.st.H, cv.used, kMinBinBytes,
		               (size_t) SRP_GPU_FIXED_SCRATCH_BYTES);
		return -1;
	}
	/* the rest: a quarter for barycentric tables, the others for tile entries */
	const size_t rest = (size_t) SRP_GPU_FIXED_SCRATCH_BYTES - cv.used;
	const size_t tableBytes = (rest / 4) & ~(size_t) 255;
	const size_t oTable = cv.take(tableBytes);
	const size_t binRoom = (size_t) SRP_GPU_FIXED_SCRATCH_BYTES - cv.used;
	const bool lineFrags = info.kind == kKindLineFrag;
	size_t entryCap = std::min<size_t>(binRoom / (16 + (lineFrags ? kRunFrags * (sizeof(LineFrag) + 4) + 1 : 0) + 2),
	                                   lineFrags ? (size_t) kMaxLineEntries : (size_t) 0xF0000000u);
	while (entryCap > 0 && binBytes(entryCap, lineFrags) > binRoom) entryCap -= entryCap / 64 + 1;
	const size_t oKeys = cv.take(entryCap * 4);
	const size_t oVals = cv.take(entryCap * 4);
	const size_t oKeys2 = cv.take(entryCap * 4);
	const size_t oVals2 = cv.take(entryCap * 4);
	const size_t oFrags = lineFrags ? cv.take(entryCap * kRunFrags * sizeof(LineFrag)) : 0;
	const size_t oFragVals = lineFrags ? cv.take(entryCap * kRunFrags * 4) : 0;
	const size_t oRunSums = lineFrags ? cv.take((size_t) runSumWords((uint32_t) entryCap) * 4) : 0;
	const size_t oHist = cv.take(sortHistWords((uint32_t) std::max<size_t>(entryCap, 1)) * 4);
	const size_t oPartials = cv.take(sortPartialWords((uint32_t) std::max<size_t>(entryCap, 1)) * 4 + 64);
	if (cv.used > (size_t) SRP_GPU_FIXED_SCRATCH_BYTES) {
		fixedDrawError(kFn, "Internal error: fixed scratch layout of %zu bytes exceeds the array", cv.used);
		return -1;
	}

	P.ctr = (DeviceCounters*) (base + oCtr);
	P.minmax = (unsigned long long*) (base + oMinmax);
	P.lookback = (unsigned long long*) (base + oLook);
	P.clip = (float4*) (base + oClip);
	P.vset0 = (float4*) (base + oSet0);
	P.vset1 = (float4*) (base + oSet1);
	P.codes = (uint8_t*) (base + oCodes);
	P.vary = (uint32_t*) (base + oVary);
	P.clipBase = (uint32_t) nV;
	P.clipCap = (uint32_t) kClipRows;
	P.clipSlot = (uint32_t*) (base + oSlot);
	P.clipPolys = (uint32_t*) (base + oPolys);
	P.clipPolyCap = (uint32_t) kClipPolys;
	if (info.kind == kKindTri) {
		P.triR = (TriRaster*) (base + oPrimA);
		P.triA = (TriAttr*) (base + oPrimB);
		P.clipFan = (uint2*) (base + oFan);
		P.clipR = (TriRaster*) (base + oFanR);
		P.clipA = (TriAttr*) (base + oFanA);
	} else if (info.kind == kKindPoint) {
		P.points = (PointRec*) (base + oPrimA);
	} else {
		P.lines = (LineRec*) (base + oPrimA);
		P.frags = (LineFrag*) (base + oFrags);
	}
	P.primCap = (uint32_t) primCap;
	P.fragCap = lineFrags ? (unsigned long long) entryCap * kRunFrags : 0;
	if (lineFrags) {
		P.fragVals = (uint32_t*) (base + oFragVals);
		P.runSums = (uint32_t*) (base + oRunSums);
	}
	P.bigJobs = (uint4*) (base + oBig);
	P.bigCap = (uint32_t) bigCap;
	P.table = (float*) (base + oTable);
	P.tableCap = tableBytes / 4;
	P.keys = (uint32_t*) (base + oKeys);
	P.vals = (uint32_t*) (base + oVals);
	P.entryCap = (uint32_t) entryCap;
	P.tileStart = (uint32_t*) (base + oStart);
	P.tileEnd = (uint32_t*) (base + oEnd);
	P.winner = (int32_t*) (base + oWinner);

	if (info.coherent) fixedDrawUpload(fb);
	/* what must start at zero: the counters (the fragment total included,
	 * since the array is shared with earlier calls) and the look-back flags;
	 * the tile ranges and the sort's histograms are cleared further down */
	cudaMemsetAsync(P.ctr, 0, sizeof(DeviceCounters), s);
	cudaMemsetAsync(P.lookback, 0, blocks * 8, s);
	launchReset(P, s);
	if (ib) launchIndexRange(P, s);
	if (ib) launchVertex(P, 0, nV, s);
	else launchVertex(P, startIndex, count, s);
	if (info.triangles) launchClipPrepass(P, s);
	launchSetup(P, s);
	unsigned launches = 3 + (ib ? 1 : 0) + (info.triangles ? 1 : 0);
	if (!launchedOk("launch")) return -1;
	cudaMemcpyAsync(&hostCounters, P.ctr, sizeof(DeviceCounters), cudaMemcpyDeviceToHost, s);
	const cudaError_t se = cudaStreamSynchronize(s);
	if (se != cudaSuccess) {
		fixedDrawError(kFn, "kernel execution: %s", cudaGetErrorString(se));
		return -1;
	}
	const DeviceCounters c = hostCounters;
	if (c.errors & kErrBadIndex) {
		fixedDrawError(kFn, "Vertex index out of range of the vertex buffer (%zu vertices)", nV);
		return -1;
	}
	if (c.errors & kErrSpin) { fixedDrawError(kFn, "Ordered-compaction wait timed out"); return -1; }
	/* sizes counted by the setup stage; any count above its room means the
	 * kernels dropped what did not fit, and nothing has been drawn yet */
	struct { const char* what; unsigned long long n; size_t room; } need[] = {
		{ "vertices created by clipping", c.clipVerts, kClipRows },
		{ "triangles that need clipping", c.clipTris, kClipPolys },
		{ "primitives", c.prims, primCap },
		{ "tile entries", c.entries, entryCap },
		{ "large primitives", c.bigJobs, bigCap },
		{ "barycentric table words", c.tableWords, P.tableCap },
	};
	for (const auto& n : need)
		if (n.n > n.room) {
			fixedDrawError(kFn, "Draw too large for the fixed scratch: %llu %s, room for %zu; nothing was drawn",
			               n.n, n.what, n.room);
			return -1;
		}
	if (c.errors & kErrCapacity) { fixedDrawError(kFn, "Fixed scratch capacity exceeded; nothing was drawn"); return -1; }

	const uint32_t E = (uint32_t) c.entries;
	/* the rest of the draw takes its sizes from the counters on the device */
	if (lineFrags) { launchLineFrags(P, s); launches += 2; }
	else if (c.bigJobs) {
		launchBigEntries(P, (uint32_t) c.bigJobs, s);
		launchLambdaTables(P, (uint32_t) c.bigJobs, s);
		launches += 2;
	}
	if (E) {
		const uint32_t keyBits = sortKeyBits(info.numTiles);
		uint32_t* sk;
		uint32_t* sv;
		sortEntries(P, keyBits, (uint32_t*) (base + oKeys2), (uint32_t*) (base + oVals2), (uint32_t*) (base + oHist),
		            (uint32_t*) (base + oPartials), &sk, &sv, s);
		launches += 1 + keyBits / 8;
		cudaMemsetAsync(P.tileStart, 0, (size_t) info.numTiles * 4, s);
		cudaMemsetAsync(P.tileEnd, 0, (size_t) info.numTiles * 4, s);
		if (lineFrags) {
			/* the sorted runs back to fragments, with their tile ranges */
			launchRunExpand(P, sk, sv, info.numTiles, s);
			sv = P.fragVals;
			launches += 2;
		} else {
			launchTileRanges(P, sk, info.numTiles, s);
		}
		if (info.late) {
			launchResolveLate(P, info.kind, sv, info.numTiles, s);
			launches += 2;
		} else {
			launchResolve(P, info.kind, sv, info.numTiles, (uint32_t*) (base + oHeavy), s);
			launchShade(P, info.kind, info.numTiles, s);
			launches += 5;
		}
	}
	const bool ok = launchedOk("launch");
	fixedDrawAccount(c, launches);
	if (info.coherent) fixedDrawDownload(fb);
	return ok ? 0 : -1;
}
