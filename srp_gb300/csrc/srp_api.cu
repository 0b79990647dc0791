/* Host side of the GPU library: the srp public API (include/srp/*.h) on top
 * of device-resident buffers, plus the additions in srp/gpu.h.
 *
 * Behaviour kept from kitrofimov/srp:
 *   state setters and defaults          src/core/context.c:15-180
 *   error reporting through the callback src/utils/message_callback.c:18-35
 *   draw validation and dispatch        src/pipeline/draw.c:63-208
 *   excess-vertex warnings              src/pipeline/primitive_assembly.c:137-153
 *   buffers (copy on CopyData)          src/core/buffer.c:20-136
 *   framebuffer clear semantics         src/core/framebuffer.c:17-62
 *   textures (3 channels, nearest)      src/core/texture.c:21-139
 * Every draw is executed by the CUDA pipeline in k_front.cu, k_bin.cu and
 * k_raster.cu; nothing is rendered on the host. */
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "srp/srp.h"
#include "srp/gpu.h"
#include "srp/mat.h"
#include "srp/shaderlib.h"
#include "gpu_types.h"
#include "imageio.h"
#include "kernels.h"
#include "draw_internal.h"
#include "learned_internal.h"

/* The reference requires the user program to define `SRPContext srpContext`.
 * A weak default lets the library also be used from programs (and language
 * bindings) that do not; a user definition takes precedence. */
extern "C" {
__attribute__((weak)) SRPContext srpContext;
}

using namespace srpg;

/* ------------------------------------------------------------- messages */

static void message(SRPMessageType type, SRPMessageSeverity sev, const char* fn, const char* fmt, ...)
{
	if (!srpContext.messageCallback.func) return;
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	srpContext.messageCallback.func(type, sev, fn, buf, srpContext.messageCallback.userParameter);
}

#define SRP_ERROR(fn, ...) message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, fn, __VA_ARGS__)

static bool cudaOk(cudaError_t e, const char* fn, const char* what)
{
	if (e == cudaSuccess) return true;
	SRP_ERROR(fn, "CUDA error in %s: %s", what, cudaGetErrorString(e));
	return false;
}

/* --------------------------------------------------------- library state */

namespace {

struct DeviceBuffer {
	void* ptr = nullptr;
	size_t bytes = 0;
	bool reserve(size_t need, const char* fn)
	{
		if (need <= bytes) return true;
		size_t nb = std::max(need, bytes + bytes / 2);
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		bytes = 0;
		if (!cudaOk(cudaMalloc(&ptr, nb), fn, "cudaMalloc")) return false;
		bytes = nb;
		return true;
	}
	template <class T> T* as() const { return (T*) ptr; }
};

struct Registry {
	std::vector<std::pair<void*, int>> vs, fs;
};

/* What one draw's resolve and shading read, written by its front stages:
 * two sets alternate between consecutive single draws, so that the front of
 * draw N+1 can run while draw N resolves and shades. A set's next front
 * waits for rasterDone, recorded after the back of the draw that used it.
 * The winner plane is per set too, so that draw N+1's resolve can run
 * while draw N's shading still reads draw N's winners. */
struct DrawSet {
	DeviceBuffer ctr, tileStart, tileEnd, heavy, vary, triR, triA, points, lines, frags, table, winner;
	/* line draws: the runs' block sums, and the fragments in sorted order */
	DeviceBuffer runSums, fragVals;
	/* the big-primitive list: written by setup, read by the binning and by
	 * the lambda tables, which run on another stream than the next front */
	DeviceBuffer big;
	/* used by the front stages only, which run on the set's own front
	 * stream: the next draw's front (other set) runs beside this one's */
	DeviceBuffer clip, vset0, vset1, codes, lookback, hist, partials, minmax, clipSlot, clipPolys;
	/* filled triangles: the fans set up by the clip pre-pass, read by setup */
	DeviceBuffer clipFan, clipR, clipA;
	cudaStream_t front = nullptr;
	DeviceBuffer keys, vals, keys2, vals2;
	/* multi-draw passes: descriptors, prefix sums, primitive bases, winners */
	DeviceBuffer passDesc, passPrefix, passPrimPrefix, passWinner;
	DeviceCounters* hostCtr = nullptr;
	cudaEvent_t ctrEvent = nullptr;    /* recorded after the counters are copied to hostCtr */
	cudaEvent_t headDone = nullptr;    /* vertex and setup done (front stream) */
	cudaEvent_t binDone = nullptr;     /* front stages done (front stream) */
	cudaEvent_t rasterDone = nullptr;  /* resolve and shade done (`stream`) */
	cudaEvent_t resolved = nullptr;    /* resolve done (resolve stream) */
};

struct Lib {
	bool init = false;
	cudaStream_t stream = nullptr;
	cudaStream_t ownStream = nullptr;
	/* heavy-tile resolve runs here, beside the light tiles on `stream` */
	cudaStream_t auxStream = nullptr;
	cudaEvent_t forkEvent = nullptr, joinEvent = nullptr;
	/* a draw's vertex, setup and binning run on its scratch set's front
	 * stream, so that the next draw's front (other set) runs beside them and
	 * beside this draw's resolve and shading */
	/* with overlap, a single draw's lambda tables and resolve run on
	 * resolveStream and its shading on `stream`: draw N+1's resolve then runs
	 * beside draw N's shading (the resolve never reads colour, the shading
	 * writes nothing else). rsDirty: `stream` holds framebuffer work queued
	 * outside a draw's shading (clear, fill, copies, passes, fixed-scratch and
	 * late-depth draws), which the next resolve on resolveStream must wait for. */
	cudaStream_t resolveStream = nullptr;
	bool rsDirty = true;
	cudaEvent_t rsEvent = nullptr;
	/* vertex and index uploads run on copyStream, so that neither the
	 * resolves nor the shading wait for uploads of later draws. A stage that
	 * reads a buffer waits for the buffer's upload event. An upload itself
	 * waits for nothing (copyStreamReady). */
	cudaStream_t copyStream = nullptr;
	unsigned long long uploadSeq = 0;
	/* srpGpuFramebufferSyncAsync copies on downloadStream, after the event of
	 * the draw or pass that last wrote the framebuffer (one of writeEvents,
	 * recorded on `stream` after its shading, numbered by writeSeq), so that
	 * a batch's first framebuffers come back while later passes render.
	 * Each download is marked by one of downloadEvents (numbered by
	 * downloadSeq); work queued later on `stream` that touches the same
	 * framebuffer first waits for its download (fbAfterDownloads), work on
	 * other framebuffers does not. streamDownloadSeq: the downloads `stream`
	 * has waited for, in order. */
	static constexpr int kWriteEvents = 64;
	cudaStream_t downloadStream = nullptr;
	cudaEvent_t writeEvents[kWriteEvents] = {};
	cudaEvent_t downloadEvents[kWriteEvents] = {};
	int writeNext = 0, downloadNext = 0;
	unsigned long long writeSeq = 0, downloadWaitedSeq = 0, downloadSeq = 0, streamDownloadSeq = 0;
	/* gathered transfers (the Batch calls): one kernel per group of buffers,
	 * item lists staged in gatherUp / gatherDown; a group's uploads end at
	 * one of gatherEvents, which its buffers borrow as their upload event */
	static constexpr int kGatherEvents = 64;
	cudaEvent_t gatherEvents[kGatherEvents] = {};
	int gatherNext = 0;
	DeviceBuffer gatherUp, gatherDown;
	bool pageableAccess = false;      /* the device reaches any host memory */
	bool overlap = true;
	bool graphs = true;               /* replay repeated draws from captured CUDA graphs */
	SRPGpuTuning tune = { 96, 3 };    /* heavy-tile threshold, heavy-tile CTAs per SM */
	SRPGpuFramebufferMode fbMode = SRP_GPU_FB_COHERENT;
	Registry reg;
	/* scratch pools, grown on demand */

	DeviceBuffer fillTargets;   /* srpGpuFramebufferFillBatch */
	DrawSet sets[2];            /* alternating between consecutive single draws */
	int setNext = 0;
	/* the frame autotuner's start event, recorded by the next draw */
	cudaEvent_t tuneStart = nullptr;
	bool tuneArmed = false;
	SRPGpuStats stats = {};
	unsigned long long launches = 0;
	uint32_t clipRows = 4096;
	uint32_t bigCap = 1 << 16;
	/* stage profiling */
	bool profiling = false;
	std::vector<cudaEvent_t> eventPool;
	std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
	SRPGpuProfile profile = {};
	cudaEvent_t openEvent = nullptr;
	unsigned long long tableCap = 1ull << 22;  /* floats */
	uint32_t clipPolyCap = 1 << 14;
	/* (tile, item) pairs per input primitive seen last, per kind of item
	 * (triangle, line fragment, point): sizes the pair buffers of the next
	 * draw of that kind, whose count the host does not wait for */
	double entryRatio[3] = { 4.0, 64.0, 4.0 };
	uint32_t bigJobsSeen[3] = { 1024, 0, 1024 };   /* big primitives of the last draw, per kind */
	/* failure-detection tests: polls before a bounded device wait gives up
	 * (0 = the kernels' default) and the signals withheld from them */
	uint32_t spinLimit = 0, waitTest = 0;
	/* the parts of a draw whose framebuffer tiles move by TMA (kTma* bits),
	 * where the planes allow it; none by default: on the 1080p soup frame
	 * every selection measured slower than direct access (8 x 8 tiles are
	 * small copies, and the resolve's staging lowers its occupancy) */
	uint32_t tma = 0;
};

Lib g;

static void syncFronts()
{
	for (DrawSet& S : g.sets)
		if (S.front) cudaStreamSynchronize(S.front);
}

bool ensureInit(const char* fn)
{
	if (g.init) return true;
	if (!cudaOk(cudaStreamCreateWithFlags(&g.ownStream, cudaStreamNonBlocking), fn, "cudaStreamCreate")) return false;
	g.stream = g.ownStream;
	int loPri = 0, hiPri = 0;
	cudaDeviceGetStreamPriorityRange(&loPri, &hiPri);
	if (!cudaOk(cudaStreamCreateWithPriority(&g.auxStream, cudaStreamNonBlocking, hiPri), fn, "cudaStreamCreate") ||
	    !cudaOk(cudaEventCreateWithFlags(&g.forkEvent, cudaEventDisableTiming), fn, "cudaEventCreate") ||
	    !cudaOk(cudaEventCreateWithFlags(&g.joinEvent, cudaEventDisableTiming), fn, "cudaEventCreate") ||
	    !cudaOk(cudaStreamCreateWithFlags(&g.sets[0].front, cudaStreamNonBlocking), fn, "cudaStreamCreate") ||
	    !cudaOk(cudaStreamCreateWithFlags(&g.sets[1].front, cudaStreamNonBlocking), fn, "cudaStreamCreate") ||
	    /* high priority: when frames are queued back to back, a frame's
	     * resolve goes ahead of the next frame's front stages */
	    !cudaOk(cudaStreamCreateWithPriority(&g.resolveStream, cudaStreamNonBlocking, hiPri), fn, "cudaStreamCreate") ||
	    !cudaOk(cudaEventCreateWithFlags(&g.rsEvent, cudaEventDisableTiming), fn, "cudaEventCreate") ||
	    !cudaOk(cudaStreamCreateWithFlags(&g.copyStream, cudaStreamNonBlocking), fn, "cudaStreamCreate") ||
	    !cudaOk(cudaStreamCreateWithFlags(&g.downloadStream, cudaStreamNonBlocking), fn, "cudaStreamCreate")) return false;
	for (cudaEvent_t& e : g.writeEvents)
		if (!cudaOk(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), fn, "cudaEventCreate")) return false;
	for (cudaEvent_t& e : g.downloadEvents)
		if (!cudaOk(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), fn, "cudaEventCreate")) return false;
	for (cudaEvent_t& e : g.gatherEvents)
		if (!cudaOk(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), fn, "cudaEventCreate")) return false;
	{
		int dev = 0, pageable = 0;
		cudaGetDevice(&dev);
		if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) cudaGetLastError();
		g.pageableAccess = pageable != 0;
	}
	for (DrawSet& S : g.sets) {
		if (!cudaOk(cudaEventCreateWithFlags(&S.ctrEvent, cudaEventDisableTiming), fn, "cudaEventCreate") ||
		    !cudaOk(cudaEventCreateWithFlags(&S.headDone, cudaEventDisableTiming), fn, "cudaEventCreate") ||
		    !cudaOk(cudaEventCreateWithFlags(&S.binDone, cudaEventDisableTiming), fn, "cudaEventCreate") ||
		    !cudaOk(cudaEventCreateWithFlags(&S.rasterDone, cudaEventDisableTiming), fn, "cudaEventCreate") ||
		    !cudaOk(cudaEventCreateWithFlags(&S.resolved, cudaEventDisableTiming), fn, "cudaEventCreate") ||
		    !cudaOk(cudaMallocHost((void**) &S.hostCtr, sizeof(DeviceCounters)), fn, "cudaMallocHost") ||
		    !S.ctr.reserve(sizeof(DeviceCounters), fn)) return false;
		memset(S.hostCtr, 0, sizeof(DeviceCounters));
		cudaMemset(S.ctr.ptr, 0, sizeof(DeviceCounters));
	}
	for (DrawSet& S : g.sets)
		if (!S.minmax.reserve(16, fn)) return false;
	g.init = true;
	return true;
}

cudaEvent_t takeEvent()
{
	if (!g.eventPool.empty()) { cudaEvent_t e = g.eventPool.back(); g.eventPool.pop_back(); return e; }
	cudaEvent_t e = nullptr;
	cudaEventCreate(&e);
	return e;
}

/* Marks the start of a stage; stageEnd records the matching event. */
void stageBegin()
{
	if (!g.profiling) return;
	g.openEvent = takeEvent();
	cudaEventRecord(g.openEvent, g.stream);
}

void stageEnd(int stage, int launches)
{
	if (!g.profiling || !g.openEvent) return;
	cudaEvent_t e = takeEvent();
	cudaEventRecord(e, g.stream);
	g.pending.push_back({ stage, { g.openEvent, e } });
	g.profile.launches[stage] += (uint64_t) launches;
	g.openEvent = nullptr;
}

/* Repeated draws replay CUDA graphs. A draw's work after its host-side
 * preparation is two fixed sequences of launches: the head (reset up to the
 * check kernel) and the tail (binning, sort, resolve, shade). Both depend
 * only on the draw parameters and a few launch sizes, which together form
 * the key; between the two the host copies the counters out directly. The
 * cache keeps the most recent kGraphCache keys. */
constexpr size_t kGraphCache = 64;

struct GraphEntry {
	std::vector<unsigned char> key;
	cudaGraphExec_t head = nullptr, head2 = nullptr, mid = nullptr, bin = nullptr, resolve = nullptr, shade = nullptr;
};

std::vector<GraphEntry> graphCache;
size_t graphNext = 0;

GraphEntry* graphFind(const std::vector<unsigned char>& key)
{
	for (auto& e : graphCache)
		if (e.key.size() == key.size() && memcmp(e.key.data(), key.data(), key.size()) == 0) return &e;
	return nullptr;
}

/* Captures `enqueue` on stream s; null if the capture failed (the caller
 * then launches directly). */
template <class F> cudaGraphExec_t captureGraph(cudaStream_t s, F&& enqueue)
{
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaGetLastError(); return nullptr; }
	enqueue();
	const cudaError_t e = cudaStreamEndCapture(s, &graph);
	if (e != cudaSuccess || !graph || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
	if (graph) cudaGraphDestroy(graph);
	cudaGetLastError();
	return exec;
}

/* Runs a draw as six sequences:
 * - head and head2: reset up to the check kernel, on the front stream `fs`,
 *   split so that `between` (an upload the second part needs) can be waited
 *   for in the middle;
 * - mid: work that needs the head but not the binning (the lambda tables),
 *   on the resolve stream `rs`, beside the bin;
 * - bin: binning and sort, on `fs`;
 * - resolve, on `rs`;
 * - shade, on the library's stream (absent for late-depth draws, whose
 *   resolve runs the shaders).
 * With fs != rs, mid waits for the head through the set's headDone event and
 * resolve for the bin through binDone; with rs != stream, shade waits for the
 * resolve through the set's resolved event, and the first work on rs waits
 * for framebuffer work queued on the library's stream since (rsDirty). The
 * shade records rasterDone. Between head and bin the counters are copied to
 * the set's host mirror. Each sequence replays its captured CUDA graph when
 * graphs are on and stage profiling is off (profiling records fresh events
 * per draw, and keeps every sequence on the library's stream). */
template <class H, class H2, class M, class B, class R, class SH>
void runDrawSeq(const std::vector<unsigned char>& key, DrawSet& S, cudaStream_t fs, cudaStream_t rs, H&& head,
                cudaEvent_t between, H2&& head2, bool hasMid, M&& mid, B&& bin, R&& resolve, bool hasShade, SH&& shade)
{
	GraphEntry* e = nullptr;
	if (g.graphs && !g.profiling) {
		e = graphFind(key);
		if (!e) {
			GraphEntry fresh;
			fresh.key = key;
			fresh.head = captureGraph(fs, head);
			fresh.head2 = fresh.head ? captureGraph(fs, head2) : nullptr;
			fresh.mid = fresh.head2 && hasMid ? captureGraph(rs, mid) : nullptr;
			fresh.bin = fresh.head2 && (fresh.mid || !hasMid) ? captureGraph(fs, bin) : nullptr;
			fresh.resolve = fresh.bin ? captureGraph(rs, resolve) : nullptr;
			fresh.shade = fresh.resolve && hasShade ? captureGraph(g.stream, shade) : nullptr;
			if (graphCache.size() < kGraphCache) graphCache.push_back(std::move(fresh));
			else {
				GraphEntry& old = graphCache[graphNext++ % kGraphCache];
				for (cudaGraphExec_t x : { old.head, old.head2, old.mid, old.bin, old.resolve, old.shade })
					if (x) cudaGraphExecDestroy(x);
				old = std::move(fresh);
			}
			e = graphFind(key);
		}
		if (e && !(e->head && e->head2 && (e->mid || !hasMid) && e->bin && e->resolve && (e->shade || !hasShade)))
			e = nullptr;
	}
	if (e) cudaGraphLaunch(e->head, fs);
	else head();
	/* an input the second part of the head needs, uploaded meanwhile */
	if (between) cudaStreamWaitEvent(fs, between, 0);
	if (e) cudaGraphLaunch(e->head2, fs);
	else head2();
	cudaMemcpyAsync(S.hostCtr, S.ctr.ptr, sizeof(DeviceCounters), cudaMemcpyDeviceToHost, fs);
	cudaEventRecord(S.ctrEvent, fs);
	if (rs != g.stream && g.rsDirty) {
		cudaEventRecord(g.rsEvent, g.stream);
		cudaStreamWaitEvent(rs, g.rsEvent, 0);
		g.rsDirty = false;
	}
	if (hasMid) {
		if (fs != rs) {
			cudaEventRecord(S.headDone, fs);
			cudaStreamWaitEvent(rs, S.headDone, 0);
		}
		if (e) cudaGraphLaunch(e->mid, rs);
		else mid();
	}
	if (e) cudaGraphLaunch(e->bin, fs);
	else bin();
	if (fs != rs) {
		cudaEventRecord(S.binDone, fs);
		cudaStreamWaitEvent(rs, S.binDone, 0);
	}
	if (e) cudaGraphLaunch(e->resolve, rs);
	else resolve();
	if (rs != g.stream) {
		cudaEventRecord(S.resolved, rs);
		cudaStreamWaitEvent(g.stream, S.resolved, 0);
	} else {
		/* the depth and stencil planes were written on the library's stream */
		g.rsDirty = true;
	}
	if (hasShade) {
		if (e) cudaGraphLaunch(e->shade, g.stream);
		else shade();
	}
	if (fs != g.stream) cudaEventRecord(S.rasterDone, g.stream);
}

/* cuTensorMapEncodeTiled, taken from the driver through the runtime (the
 * library does not link the driver library itself); null if unavailable. */
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiledFn()
{
	static EncodeTiledFn fn = nullptr;
	static bool looked = false;
	if (!looked) {
		looked = true;
		void* p = nullptr;
		cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = (EncodeTiledFn) p;
		else
			cudaGetLastError();
	}
	return fn;
}

/* Tensor map of a W x H plane of 32-bit pixels with rows of W pixels, in
 * 8 x 8 boxes: the tile copies of the resolve and the shading. The plane
 * must start on 16 bytes and W be a multiple of 4 (16-byte row pitch). */
bool encodeTileMap(CUtensorMap* m, void* plane, int W, int H, CUtensorMapDataType type)
{
	const EncodeTiledFn fn = encodeTiledFn();
	if (!fn || !plane || W <= 0 || H <= 0 || (W & 3) || ((uintptr_t) plane & 15)) return false;
	const cuuint64_t dims[2] = { (cuuint64_t) W, (cuuint64_t) H };
	const cuuint64_t strides[1] = { (cuuint64_t) W * 4 };
	const cuuint32_t box[2] = { (cuuint32_t) kTile, (cuuint32_t) kTile };
	const cuuint32_t elem[2] = { 1, 1 };
	return fn(m, type, 2, plane, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
	          CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

/* The key of a draw: its parameters and the host-side launch sizes. */
std::vector<unsigned char> graphKey(const DrawParams& P, std::initializer_list<unsigned long long> sizes)
{
	std::vector<unsigned char> k(sizeof(DrawParams) + sizes.size() * 8);
	memcpy(k.data(), &P, sizeof(DrawParams));
	size_t o = sizeof(DrawParams);
	for (unsigned long long v : sizes) { memcpy(k.data() + o, &v, 8); o += 8; }
	return k;
}

}  // namespace

/* ---------------------------------------------------------------- context */

extern "C" {

void srpNewContext(SRPContext* c)
{
	c->messageCallback.func = NULL;
	c->messageCallback.userParameter = NULL;
	c->provokingVertexMode = SRP_PROVOKING_VERTEX_LAST;
	c->raster.frontFace = SRP_WINDING_CCW;
	c->raster.cullFace = SRP_FACE_NONE;
	c->raster.polygonMode = SRP_POLYGON_MODE_FILL;
	c->raster.pointSize = 1.f;
	memset(&c->scissor, 0, sizeof c->scissor);
	c->depth.testEnable = false;
	c->depth.writeEnable = true;
	c->depth.compareOp = SRP_COMPARE_GREATER;
	SRPStencilFaceState f = { SRP_COMPARE_ALWAYS, 0, 0xFF, 0xFF, SRP_STENCIL_KEEP, SRP_STENCIL_KEEP, SRP_STENCIL_KEEP };
	c->stencil.enabled = false;
	c->stencil.front = f;
	c->stencil.back = f;
	c->arena = NULL;
}

void srpSetMessageCallback(SRPMessageCallback cb) { srpContext.messageCallback = cb; }
void srpProvokingVertexMode(SRPProvokingVertexMode m) { srpContext.provokingVertexMode = m; }
void srpRasterCullFace(SRPFace f) { srpContext.raster.cullFace = f; }
void srpRasterFrontFace(SRPWinding w) { srpContext.raster.frontFace = w; }
void srpRasterPolygonMode(SRPPolygonMode m) { srpContext.raster.polygonMode = m; }
void srpRasterPointSize(float s) { srpContext.raster.pointSize = s; }
void srpScissorTest(bool e) { srpContext.scissor.enabled = e; }
void srpScissorOptions(size_t x, size_t y, size_t w, size_t h)
{
	srpContext.scissor.x = x; srpContext.scissor.y = y;
	srpContext.scissor.width = w; srpContext.scissor.height = h;
}
/* enables the test whatever the argument, as the reference does */
void srpStencilTest(bool) { srpContext.stencil.enabled = true; }
void srpStencilFunc(SRPCompareOp func, uint8_t ref, uint8_t mask)
{
	SRPStencilFaceState* s[2] = { &srpContext.stencil.front, &srpContext.stencil.back };
	for (auto* f : s) { f->func = func; f->ref = ref; f->mask = mask; }
}
static SRPStencilFaceState* faceState(SRPFace face)
{
	return face == SRP_FACE_FRONT ? &srpContext.stencil.front : &srpContext.stencil.back;
}
void srpStencilFuncSeparate(SRPFace face, SRPCompareOp func, uint8_t ref, uint8_t mask)
{
	if (face == SRP_FACE_NONE) return;
	if (face == SRP_FACE_FRONT_AND_BACK) srpStencilFunc(func, ref, mask);
	SRPStencilFaceState* s = faceState(face);
	s->func = func; s->ref = ref; s->mask = mask;
}
void srpStencilOp(SRPStencilOp sfail, SRPStencilOp dfail, SRPStencilOp pass)
{
	SRPStencilFaceState* s[2] = { &srpContext.stencil.front, &srpContext.stencil.back };
	for (auto* f : s) { f->sfailOp = sfail; f->dfailOp = dfail; f->passOp = pass; }
}
void srpStencilOpSeparate(SRPFace face, SRPStencilOp sfail, SRPStencilOp dfail, SRPStencilOp pass)
{
	if (face == SRP_FACE_NONE) return;
	if (face == SRP_FACE_FRONT_AND_BACK) srpStencilOp(sfail, dfail, pass);
	SRPStencilFaceState* s = faceState(face);
	s->sfailOp = sfail; s->dfailOp = dfail; s->passOp = pass;
}
void srpStencilWriteMask(uint8_t mask)
{
	srpContext.stencil.front.writeMask = mask;
	srpContext.stencil.back.writeMask = mask;
}
void srpStencilWriteMaskSeparate(SRPFace face, uint8_t mask)
{
	if (face == SRP_FACE_NONE) return;
	if (face == SRP_FACE_FRONT_AND_BACK) srpStencilWriteMask(mask);
	faceState(face)->writeMask = mask;
}
void srpDepthTest(bool e) { srpContext.depth.testEnable = e; }
void srpDepthWrite(bool e) { srpContext.depth.writeEnable = e; }
void srpDepthCompareOp(SRPCompareOp op) { srpContext.depth.compareOp = op; }

}  // extern "C"

/* ---------------------------------------------------------------- buffers */

struct SRPVertexBuffer {
	size_t stride = 0, nVertices = 0, nBytes = 0, cap = 0;
	unsigned char* host = nullptr;    /* staging copy made by CopyData */
	DeviceBuffer dev;
	bool dirty = false;
	cudaEvent_t ready = nullptr;      /* recorded after the last upload (copy stream) */
	bool readyOwned = true;           /* false: ready is a gathered group's event */
	bool pending = false;             /* uploaded since a pass's front last waited for it */
	unsigned long long seq = 0;       /* upload number of the last upload */
};

struct SRPIndexBuffer {
	SRPType type = SRP_UINT8;
	size_t elemSize = 1, nIndices = 0, nBytes = 0, cap = 0;
	unsigned char* host = nullptr;
	DeviceBuffer dev;
	bool dirty = false;
	cudaEvent_t ready = nullptr;
	bool readyOwned = true;
	bool pending = false;
	unsigned long long seq = 0;
};

/* Marks the end of an upload into a buffer: the stage of a later draw that
 * reads the buffer waits for it. Uploads are numbered in the order of the
 * copy stream, on which they complete in that order. */
static void markUpload(cudaEvent_t& ready, bool& readyOwned, bool& pending, unsigned long long& seq)
{
	if (!readyOwned) {
		ready = nullptr;
		readyOwned = true;
	}
	if (!ready && cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess) {
		cudaGetLastError();
		ready = nullptr;
		return;
	}
	cudaEventRecord(ready, g.copyStream);
	pending = true;
	seq = ++g.uploadSeq;
}

/* The stream of vertex and index uploads. An upload need not wait for the
 * draws queued before it: only the index-range, vertex, clip pre-pass and
 * setup kernels read those buffers, all of them before the draw's setup
 * counters are copied, and every draw call (single draws, multi-draw passes,
 * the fixed-scratch draw) waits on the host for those counters before it
 * returns. So when an upload is issued no earlier draw still reads the
 * buffer, and the next frame's uploads run beside this frame's resolve and
 * shading. */
static cudaStream_t copyStreamReady() { return g.copyStream; }

/* ------------------------------------------------------ gathered copies */

/* One contiguous copy of a gathered transfer, cut into kGatherChunk pieces;
 * firstChunk counts the pieces of the items before it. */
struct GatherItem {
	const unsigned char* src;
	unsigned char* dst;
	unsigned long long bytes;
	unsigned long long firstChunk;
};
constexpr unsigned long long kGatherChunk = 64ull << 10;

/* A block per piece, its item found by binary search over firstChunk.
 * Sources and destinations are device memory or host memory that the device
 * reaches (page-locked, or any host memory with pageable-memory access). */
__global__ void k_gather(const GatherItem* items, unsigned n, unsigned long long chunks)
{
	for (unsigned long long c = blockIdx.x; c < chunks; c += gridDim.x) {
		unsigned lo = 0, hi = n;
		while (hi - lo > 1) {
			const unsigned mid = (lo + hi) / 2;
			if (items[mid].firstChunk <= c) lo = mid;
			else hi = mid;
		}
		const GatherItem it = items[lo];
		const unsigned long long off = (c - it.firstChunk) * kGatherChunk;
		const unsigned long long len = it.bytes - off < kGatherChunk ? it.bytes - off : kGatherChunk;
		const unsigned char* src = it.src + off;
		unsigned char* dst = it.dst + off;
		if ((((uintptr_t) src) | ((uintptr_t) dst)) % 16 == 0) {
			const unsigned long long n16 = len / 16;
			for (unsigned long long i = threadIdx.x; i < n16; i += blockDim.x) ((uint4*) dst)[i] = ((const uint4*) src)[i];
			for (unsigned long long i = n16 * 16 + threadIdx.x; i < len; i += blockDim.x) dst[i] = src[i];
		} else {
			for (unsigned long long i = threadIdx.x; i < len; i += blockDim.x) dst[i] = src[i];
		}
	}
}

/* The address by which the device reaches host memory p, or null. */
static void* deviceView(const void* p)
{
	if (g.pageableAccess) return (void*) p;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeDevice)
		return a.devicePointer ? a.devicePointer : (void*) p;
	return nullptr;
}

/* Enqueues the copies of items [first, last) as one kernel on stream s, its
 * item list staged in dev at offset `slot` items (from pageable memory: the
 * call returns once the list has been read). */
static bool gatherLaunch(std::vector<GatherItem>& items, size_t first, size_t last, DeviceBuffer& dev, size_t slot,
                         cudaStream_t s, const char* fn)
{
	if (last <= first) return true;
	unsigned long long chunks = 0;
	for (size_t i = first; i < last; ++i) {
		items[i].firstChunk = chunks;
		chunks += (items[i].bytes + kGatherChunk - 1) / kGatherChunk;
	}
	GatherItem* d = dev.as<GatherItem>() + slot;
	if (!cudaOk(cudaMemcpyAsync(d, items.data() + first, (last - first) * sizeof(GatherItem), cudaMemcpyHostToDevice, s),
	            fn, "cudaMemcpyAsync")) return false;
	const unsigned blocks = (unsigned) std::min<unsigned long long>(chunks, 256);
	k_gather<<<blocks, 256, 0, s>>>(d, (unsigned) (last - first), chunks);
	++g.launches;
	return cudaOk(cudaGetLastError(), fn, "launch");
}

static size_t indexTypeSize(SRPType t)
{
	/* srpSizeofType (src/utils/type.c:15-40) */
	switch (t) {
	case SRP_UINT8: return 1;
	case SRP_UINT16: return 2;
	case SRP_UINT32: case SRP_FLOAT: return 4;
	case SRP_UINT64: case SRP_DOUBLE: return 8;
	default:
		SRP_ERROR("srpSizeofType", "Unknown type (%i)", (int) t);
		return 0;
	}
}

/* True when a CUDA device is usable (probed once, silently). */
static bool gpuPresent()
{
	static int present = -1;
	if (present < 0) {
		int n = 0;
		present = cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
	}
	return present == 1;
}

/* CopyData on a machine with a GPU: the bytes go straight to HBM, on the
 * library's copy stream, and the copy is waited for before returning (the
 * caller may reuse its buffer at once, as with the reference's memcpy, and
 * the buffer is in device memory for any later work). */
static bool copyToDevice(DeviceBuffer& dev, const void* data, size_t nBytes, const char* fn)
{
	if (!ensureInit(fn) || !dev.reserve(nBytes + 16, fn)) return false;
	if (!nBytes) return true;
	const cudaStream_t cs = copyStreamReady();
	if (!cudaOk(cudaMemcpyAsync(dev.ptr, data, nBytes, cudaMemcpyHostToDevice, cs), fn, "cudaMemcpyAsync")) return false;
	return cudaOk(cudaStreamSynchronize(cs), fn, "cudaMemcpyAsync");
}

/* CopyData without the wait: the copy is only enqueued on the copy stream,
 * and the caller keeps `data` unchanged until srpGpuSynchronize. */
static bool copyToDeviceAsync(DeviceBuffer& dev, const void* data, size_t nBytes, const char* fn)
{
	if (!ensureInit(fn) || !dev.reserve(nBytes + 16, fn)) return false;
	if (!nBytes) return true;
	return cudaOk(cudaMemcpyAsync(dev.ptr, data, nBytes, cudaMemcpyHostToDevice, copyStreamReady()), fn,
	              "cudaMemcpyAsync");
}

static void* pinnedRealloc(void* old, size_t n)
{
	if (old) cudaFreeHost(old);
	void* p = nullptr;
	if (cudaMallocHost(&p, n ? n : 1) != cudaSuccess) {
		p = malloc(n ? n : 1);
		if (!p) { fprintf(stderr, "srp-gb300: out of host memory\n"); abort(); }
	}
	return p;
}

extern "C" {

SRPVertexBuffer* srpNewVertexBuffer(void) { return new SRPVertexBuffer(); }

void srpFreeVertexBuffer(SRPVertexBuffer* b)
{
	if (!b) return;
	if (g.init) cudaStreamSynchronize(g.copyStream);  /* copies from b->host may be in flight */
	if (b->ready && b->readyOwned) cudaEventDestroy(b->ready);
	if (b->host) cudaFreeHost(b->host);
	if (b->dev.ptr) cudaFree(b->dev.ptr);
	delete b;
}

void srpVertexBufferCopyData(SRPVertexBuffer* b, size_t stride, size_t nBytes, const void* data)
{
	b->stride = stride;
	b->nVertices = stride ? nBytes / stride : 0;
	b->nBytes = nBytes;
	if (gpuPresent()) {
		b->dirty = !copyToDevice(b->dev, data, nBytes, "srpVertexBufferCopyData");
		if (!b->dirty) { markUpload(b->ready, b->readyOwned, b->pending, b->seq); return; }
	}
	/* no device: keep a host copy, uploaded by the first draw */
	if (nBytes > b->cap) { b->host = (unsigned char*) pinnedRealloc(b->host, nBytes); b->cap = nBytes; }
	if (nBytes) memcpy(b->host, data, nBytes);
	b->dirty = true;
}

void srpGpuVertexBufferCopyDataAsync(SRPVertexBuffer* b, size_t stride, size_t nBytes, const void* data)
{
	if (!gpuPresent()) { srpVertexBufferCopyData(b, stride, nBytes, data); return; }
	b->stride = stride;
	b->nVertices = stride ? nBytes / stride : 0;
	b->nBytes = nBytes;
	b->dirty = !copyToDeviceAsync(b->dev, data, nBytes, "srpGpuVertexBufferCopyDataAsync");
	if (b->dirty) srpVertexBufferCopyData(b, stride, nBytes, data);
	else markUpload(b->ready, b->readyOwned, b->pending, b->seq);
}

SRPIndexBuffer* srpNewIndexBuffer(void) { return new SRPIndexBuffer(); }

void srpFreeIndexBuffer(SRPIndexBuffer* b)
{
	if (!b) return;
	if (g.init) cudaStreamSynchronize(g.copyStream);  /* copies from b->host may be in flight */
	if (b->ready && b->readyOwned) cudaEventDestroy(b->ready);
	if (b->host) cudaFreeHost(b->host);
	if (b->dev.ptr) cudaFree(b->dev.ptr);
	delete b;
}

void srpIndexBufferCopyData(SRPIndexBuffer* b, SRPType type, size_t nBytes, const void* data)
{
	b->type = type;
	b->elemSize = indexTypeSize(type);
	/* the reference divides by zero for a type without a size; report instead */
	b->nIndices = b->elemSize ? nBytes / b->elemSize : 0;
	b->nBytes = nBytes;
	if (gpuPresent()) {
		b->dirty = !copyToDevice(b->dev, data, nBytes, "srpIndexBufferCopyData");
		if (!b->dirty) { markUpload(b->ready, b->readyOwned, b->pending, b->seq); return; }
	}
	if (nBytes > b->cap) { b->host = (unsigned char*) pinnedRealloc(b->host, nBytes); b->cap = nBytes; }
	if (nBytes) memcpy(b->host, data, nBytes);
	b->dirty = true;
}

void srpGpuIndexBufferCopyDataAsync(SRPIndexBuffer* b, SRPType type, size_t nBytes, const void* data)
{
	if (!gpuPresent()) { srpIndexBufferCopyData(b, type, nBytes, data); return; }
	b->type = type;
	b->elemSize = indexTypeSize(type);
	b->nIndices = b->elemSize ? nBytes / b->elemSize : 0;
	b->nBytes = nBytes;
	b->dirty = !copyToDeviceAsync(b->dev, data, nBytes, "srpGpuIndexBufferCopyDataAsync");
	if (b->dirty) srpIndexBufferCopyData(b, type, nBytes, data);
	else markUpload(b->ready, b->readyOwned, b->pending, b->seq);
}

/* An upload of a Batch call: the buffer's device memory, the source as the
 * device reaches it, and the buffer's upload bookkeeping. */
struct UploadTarget {
	DeviceBuffer* dev;
	const void* src;
	size_t bytes;
	cudaEvent_t* ready;
	bool* readyOwned;
	bool* pending;
	unsigned long long* seq;
	bool* dirty;
};

/* Gathered uploads, in groups of 256 buffers: one kernel per group on the
 * copy stream, and one event, which the group's buffers borrow as their
 * upload event. */
static void gatherUploads(std::vector<UploadTarget>& t, const char* fn)
{
	if (t.empty()) return;
	const cudaStream_t cs = copyStreamReady();
	std::vector<GatherItem> items;
	items.reserve(t.size());
	for (const UploadTarget& u : t) items.push_back({ (const unsigned char*) u.src, (unsigned char*) u.dev->ptr, u.bytes, 0 });
	if (!g.gatherUp.reserve(items.size() * sizeof(GatherItem), fn)) return;
	constexpr size_t kGroup = 256;
	for (size_t first = 0; first < items.size(); first += kGroup) {
		const size_t last = std::min(items.size(), first + kGroup);
		if (!gatherLaunch(items, first, last, g.gatherUp, first, cs, fn)) return;
		cudaEvent_t e = g.gatherEvents[g.gatherNext];
		g.gatherNext = (g.gatherNext + 1) % Lib::kGatherEvents;
		cudaEventRecord(e, cs);
		const unsigned long long seq = ++g.uploadSeq;
		for (size_t k = first; k < last; ++k) {
			UploadTarget& u = t[k];
			if (*u.ready && *u.readyOwned) cudaEventDestroy(*u.ready);
			*u.ready = e;
			*u.readyOwned = false;
			*u.pending = true;
			*u.seq = seq;
			*u.dirty = false;
		}
	}
}

void srpGpuVertexBufferCopyDataBatchAsync(SRPVertexBuffer* const* buffers, const size_t* strides, const size_t* nBytes,
                                          const void* const* data, size_t n)
{
	const char* FN = "srpGpuVertexBufferCopyDataBatchAsync";
	if (!n || !buffers) return;
	if (!gpuPresent() || !ensureInit(FN)) {
		for (size_t i = 0; i < n; ++i) srpVertexBufferCopyData(buffers[i], strides[i], nBytes[i], data[i]);
		return;
	}
	/* a buffer given more than once keeps its last copy, as n single calls
	 * would leave it */
	std::vector<UploadTarget> t;
	t.reserve(n);
	std::unordered_set<const SRPVertexBuffer*> seen;
	for (size_t i = n; i-- > 0;) {
		SRPVertexBuffer* b = buffers[i];
		if (!seen.insert(b).second) continue;
		const void* src = nBytes[i] ? deviceView(data[i]) : nullptr;
		if (!src || !b->dev.reserve(nBytes[i] + 16, FN)) {
			srpGpuVertexBufferCopyDataAsync(b, strides[i], nBytes[i], data[i]);
			continue;
		}
		b->stride = strides[i];
		b->nVertices = strides[i] ? nBytes[i] / strides[i] : 0;
		b->nBytes = nBytes[i];
		t.push_back({ &b->dev, src, nBytes[i], &b->ready, &b->readyOwned, &b->pending, &b->seq, &b->dirty });
	}
	std::reverse(t.begin(), t.end());
	gatherUploads(t, FN);
}

void srpGpuIndexBufferCopyDataBatchAsync(SRPIndexBuffer* const* buffers, const SRPType* types, const size_t* nBytes,
                                         const void* const* data, size_t n)
{
	const char* FN = "srpGpuIndexBufferCopyDataBatchAsync";
	if (!n || !buffers) return;
	if (!gpuPresent() || !ensureInit(FN)) {
		for (size_t i = 0; i < n; ++i) srpIndexBufferCopyData(buffers[i], types[i], nBytes[i], data[i]);
		return;
	}
	std::vector<UploadTarget> t;
	t.reserve(n);
	std::unordered_set<const SRPIndexBuffer*> seen;
	for (size_t i = n; i-- > 0;) {
		SRPIndexBuffer* b = buffers[i];
		if (!seen.insert(b).second) continue;
		const size_t elem = indexTypeSize(types[i]);
		const void* src = nBytes[i] && elem ? deviceView(data[i]) : nullptr;
		if (!src || !b->dev.reserve(nBytes[i] + 16, FN)) {
			srpGpuIndexBufferCopyDataAsync(b, types[i], nBytes[i], data[i]);
			continue;
		}
		b->type = types[i];
		b->elemSize = elem;
		b->nIndices = nBytes[i] / elem;
		b->nBytes = nBytes[i];
		t.push_back({ &b->dev, src, nBytes[i], &b->ready, &b->readyOwned, &b->pending, &b->seq, &b->dirty });
	}
	std::reverse(t.begin(), t.end());
	gatherUploads(t, FN);
}

}  // extern "C"

/* ------------------------------------------------------------ framebuffer */

namespace {
struct FbExtra {
	uint32_t* color = nullptr;
	float* depth = nullptr;
	uint8_t* stencil = nullptr;
	/* the draw or pass that last wrote the planes: its event and number
	 * (null after any other write, whose end the library's stream marks) */
	cudaEvent_t lastWrite = nullptr;
	unsigned long long lastWriteSeq = 0;
	/* its last download on the download stream: the event and number */
	cudaEvent_t download = nullptr;
	unsigned long long downloadSeq = 0;
	/* the host block of the planes as made by srpNewFramebuffer, and the
	 * address by which the device reaches it (null if it cannot) */
	void* hostBase = nullptr;
	void* hostDev = nullptr;
};
/* The public struct has no room for device pointers; they live in a side
 * table keyed by the framebuffer address. */
std::unordered_map<const SRPFramebuffer*, FbExtra> fbTable;

FbExtra* fbFind(const SRPFramebuffer* fb)
{
	auto it = fbTable.find(fb);
	return it == fbTable.end() ? nullptr : &it->second;
}
}  // namespace

__global__ void k_fill32(uint32_t* p, uint32_t v, size_t n)
{
	for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x) p[i] = v;
}

/* One framebuffer of srpGpuFramebufferFillBatch. */
struct FillTarget {
	uint32_t* color;
	uint32_t* depth;
	uint8_t* stencil;
	size_t size;
};

/* blockIdx.y strides over the framebuffers, blockIdx.x over their pixels */
__global__ void k_fill_batch(const FillTarget* t, size_t n, uint32_t color, uint32_t depth, uint8_t stencil,
                             unsigned planes)
{
	for (size_t f = blockIdx.y; f < n; f += gridDim.y) {
		const FillTarget T = t[f];
		for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < T.size; i += (size_t) gridDim.x * blockDim.x) {
			if (planes & SRP_GPU_FILL_COLOR) T.color[i] = color;
			if (planes & SRP_GPU_FILL_DEPTH) T.depth[i] = depth;
			if (planes & SRP_GPU_FILL_STENCIL) T.stencil[i] = stencil;
		}
	}
}

static void fill32(uint32_t* p, uint32_t v, size_t n)
{
	if (!n) return;
	size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 16);
	k_fill32<<<(unsigned) blocks, 256, 0, g.stream>>>(p, v, n);
	++g.launches;
}

/* The planes of a framebuffer made by srpNewFramebuffer are one block on
 * each side (colour, depth, stencil); a program may have pointed the public
 * arrays elsewhere, in which case they are copied one by one. */
static bool fbContiguous(const SRPFramebuffer* fb)
{
	const size_t n = fb->size ? fb->size : 1;
	return (unsigned char*) fb->depth == (unsigned char*) fb->color + 4 * n &&
	       fb->stencil == (unsigned char*) fb->color + 8 * n;
}

/* Work on framebuffer x about to be queued on the library's stream comes
 * after x's download on the download stream, which reads the planes into
 * the host arrays; the resolve stream follows through rsDirty. Downloads
 * complete in order, so waiting for one covers every earlier one. */
static void fbAfterDownloads(FbExtra* x)
{
	if (x->downloadSeq <= g.streamDownloadSeq) return;
	cudaStreamWaitEvent(g.stream, x->download, 0);
	g.streamDownloadSeq = x->downloadSeq;
	g.rsDirty = true;
}

/* Marks the downloads just queued on the download stream; returns the event
 * and its number. */
static cudaEvent_t downloadMark(unsigned long long& seq)
{
	cudaEvent_t e = g.downloadEvents[g.downloadNext];
	g.downloadNext = (g.downloadNext + 1) % Lib::kWriteEvents;
	cudaEventRecord(e, g.downloadStream);
	seq = ++g.downloadSeq;
	return e;
}

/* A write other than a draw's: later downloads of the framebuffer wait for
 * the library's stream. */
static void fbOtherWrite(FbExtra* x)
{
	fbAfterDownloads(x);
	x->lastWrite = nullptr;
}

/* The end of a draw or pass, marked on the library's stream after its
 * shading; returns the event and its number. */
static cudaEvent_t drawWriteEvent(unsigned long long& seq)
{
	cudaEvent_t e = g.writeEvents[g.writeNext];
	g.writeNext = (g.writeNext + 1) % Lib::kWriteEvents;
	cudaEventRecord(e, g.stream);
	seq = ++g.writeSeq;
	return e;
}

static void fbUpload(const SRPFramebuffer* fb, FbExtra* x)
{
	fbOtherWrite(x);
	g.rsDirty = true;
	if (fbContiguous(fb)) {
		cudaMemcpyAsync(x->color, fb->color, 9 * fb->size, cudaMemcpyHostToDevice, g.stream);
		return;
	}
	cudaMemcpyAsync(x->color, fb->color, 4 * fb->size, cudaMemcpyHostToDevice, g.stream);
	cudaMemcpyAsync(x->depth, fb->depth, 4 * fb->size, cudaMemcpyHostToDevice, g.stream);
	cudaMemcpyAsync(x->stencil, fb->stencil, fb->size, cudaMemcpyHostToDevice, g.stream);
}

static void fbDownloadAsync(const SRPFramebuffer* fb, FbExtra* x)
{
	fbAfterDownloads(x);  /* the same host arrays */
	g.rsDirty = true;
	if (fbContiguous(fb)) {
		cudaMemcpyAsync(fb->color, x->color, 9 * fb->size, cudaMemcpyDeviceToHost, g.stream);
		return;
	}
	cudaMemcpyAsync(fb->color, x->color, 4 * fb->size, cudaMemcpyDeviceToHost, g.stream);
	cudaMemcpyAsync(fb->depth, x->depth, 4 * fb->size, cudaMemcpyDeviceToHost, g.stream);
	cudaMemcpyAsync(fb->stencil, x->stencil, fb->size, cudaMemcpyDeviceToHost, g.stream);
}

static void fbDownload(const SRPFramebuffer* fb, FbExtra* x)
{
	fbDownloadAsync(fb, x);
	cudaStreamSynchronize(g.stream);
}

extern "C" {

SRPFramebuffer* srpNewFramebuffer(size_t w, size_t h)
{
	if (!ensureInit("srpNewFramebuffer")) return nullptr;
	if (w > 32767 || h > 32767) {
		SRP_ERROR("srpNewFramebuffer", "Framebuffer %zux%zu exceeds the GPU limit of 32767 per side", w, h);
		return nullptr;
	}
	SRPFramebuffer* fb = (SRPFramebuffer*) calloc(1, sizeof(SRPFramebuffer));
	fb->width = w; fb->height = h; fb->size = w * h;
	/* the three planes, host and device alike, are one block each:
	 * colour (4 B/px), depth (4 B/px), stencil (1 B/px), so that a sync is one copy */
	const size_t n = fb->size ? fb->size : 1;
	unsigned char* host = (unsigned char*) pinnedRealloc(nullptr, 9 * n);
	memset(host, 0, 9 * n);
	fb->color = (uint32_t*) host;
	fb->depth = (float*) (host + 4 * n);
	fb->stencil = host + 8 * n;
	FbExtra x;
	unsigned char* dev = nullptr;
	if (!cudaOk(cudaMalloc(&dev, 9 * n), "srpNewFramebuffer", "cudaMalloc")) return fb;
	x.color = (uint32_t*) dev;
	x.depth = (float*) (dev + 4 * n);
	x.stencil = dev + 8 * n;
	x.hostBase = host;
	x.hostDev = deviceView(host);
	cudaMemsetAsync(dev, 0, 9 * n, g.stream);
	g.rsDirty = true;
	fbTable[fb] = x;
	return fb;
}

void srpFreeFramebuffer(SRPFramebuffer* fb)
{
	if (!fb) return;
	if (g.init) {
		syncFronts();
		cudaStreamSynchronize(g.resolveStream);
		cudaStreamSynchronize(g.downloadStream);  /* into the host arrays freed below */
	}
	cudaStreamSynchronize(g.stream);
	auto it = fbTable.find(fb);
	if (it != fbTable.end()) {
		cudaFree(it->second.color);  /* base of the planes' block */
		fbTable.erase(it);
	}
	cudaFreeHost(fb->color);  /* base of the planes' block */
	free(fb);
}

void srpFramebufferClear(const SRPFramebuffer* fb)
{
	FbExtra* x = fbFind(fb);
	if (!x) return;
	fbOtherWrite(x);
	g.rsDirty = true;
	cudaMemsetAsync(x->color, 0, 4 * fb->size, g.stream);
	fill32((uint32_t*) x->depth, 0xBF800000u /* -1.0f */, fb->size);
	if (g.fbMode == SRP_GPU_FB_COHERENT) {
		memset(fb->color, 0, 4 * fb->size);
		for (size_t i = 0; i < fb->size; ++i) fb->depth[i] = -1.0f;
	}
}

void srpGpuSetFramebufferMode(SRPGpuFramebufferMode mode) { g.fbMode = mode; }
SRPGpuFramebufferMode srpGpuGetFramebufferMode(void) { return g.fbMode; }

void srpGpuFramebufferSync(const SRPFramebuffer* fb)
{
	FbExtra* x = fbFind(fb);
	if (x) fbDownload(fb, x);
}

int srpGpuSaveFramebufferPNG(const SRPFramebuffer* fb, const char* path)
{
	const char* FN = "srpGpuSaveFramebufferPNG";
	if (!fb || !path) return 1;
	FbExtra* x = fbFind(fb);
	if (!x) { SRP_ERROR(FN, "Framebuffer was not created by srpNewFramebuffer"); return 1; }
	/* the host planes are current in the coherent mode (and may hold the
	 * program's own edits); in the device mode they are refreshed first */
	if (g.fbMode == SRP_GPU_FB_DEVICE) fbDownload(fb, x);
	/* as the reference's test harness saves images: R, G, B from the packed
	 * colour, alpha 255 (tests/utils/save.c:3-34) */
	std::vector<uint8_t> rgba(fb->size * 4);
	for (size_t i = 0; i < fb->size; ++i) {
		const uint32_t c = fb->color[i];
		rgba[4 * i + 0] = (uint8_t) (c >> 24);
		rgba[4 * i + 1] = (uint8_t) (c >> 16);
		rgba[4 * i + 2] = (uint8_t) (c >> 8);
		rgba[4 * i + 3] = 0xFF;
	}
	if (!srpImageWritePNG(path, rgba.data(), (int) fb->width, (int) fb->height)) {
		SRP_ERROR(FN, "Cannot write %s", path);
		return 1;
	}
	return 0;
}

void srpGpuFramebufferSyncAsync(const SRPFramebuffer* fb)
{
	FbExtra* x = fbFind(fb);
	if (!x) return;
	if (!x->lastWrite || !fbContiguous(fb)) {
		fbDownloadAsync(fb, x);
		return;
	}
	/* after the draw or pass that wrote it last, beside later ones */
	if (x->lastWriteSeq > g.downloadWaitedSeq) {
		cudaStreamWaitEvent(g.downloadStream, x->lastWrite, 0);
		g.downloadWaitedSeq = x->lastWriteSeq;
	}
	cudaMemcpyAsync(fb->color, x->color, 9 * fb->size, cudaMemcpyDeviceToHost, g.downloadStream);
	x->download = downloadMark(x->downloadSeq);
}

void srpGpuFramebufferSyncBatchAsync(const SRPFramebuffer* const* fbs, size_t n)
{
	const char* FN = "srpGpuFramebufferSyncBatchAsync";
	if (!n || !fbs) return;
	if (!g.init || !g.gatherDown.reserve(n * sizeof(GatherItem), FN)) {
		for (size_t i = 0; i < n; ++i) srpGpuFramebufferSyncAsync(fbs[i]);
		return;
	}
	/* runs of framebuffers last written by the same draw or pass: one kernel
	 * each on the download stream, after that draw or pass */
	std::vector<GatherItem> items;
	std::vector<FbExtra*> owners;
	items.reserve(n);
	owners.reserve(n);
	size_t first = 0;
	cudaEvent_t runEvent = nullptr;
	unsigned long long runSeq = 0;
	auto flush = [&]() {
		if (items.size() > first) {
			if (runSeq > g.downloadWaitedSeq) {
				cudaStreamWaitEvent(g.downloadStream, runEvent, 0);
				g.downloadWaitedSeq = runSeq;
			}
			gatherLaunch(items, first, items.size(), g.gatherDown, first, g.downloadStream, FN);
			unsigned long long seq = 0;
			const cudaEvent_t e = downloadMark(seq);
			for (size_t k = first; k < items.size(); ++k) {
				owners[k]->download = e;
				owners[k]->downloadSeq = seq;
			}
		}
		first = items.size();
	};
	for (size_t i = 0; i < n; ++i) {
		const SRPFramebuffer* fb = fbs[i];
		FbExtra* x = fbFind(fb);
		if (!x) continue;
		if (!x->lastWrite || !x->hostDev || (void*) fb->color != x->hostBase || !fbContiguous(fb) || !fb->size) {
			srpGpuFramebufferSyncAsync(fb);
			continue;
		}
		if (x->lastWriteSeq != runSeq) {
			flush();
			runEvent = x->lastWrite;
			runSeq = x->lastWriteSeq;
		}
		items.push_back({ (const unsigned char*) x->color, (unsigned char*) x->hostDev, 9ull * fb->size, 0 });
		owners.push_back(x);
	}
	flush();
}

void srpGpuFramebufferFillBatch(const SRPFramebuffer* const* fbs, size_t n, uint32_t color, float depth,
                                uint8_t stencil, unsigned planes)
{
	const char* FN = "srpGpuFramebufferFillBatch";
	if (!n || !fbs || !ensureInit(FN)) return;
	std::vector<FillTarget> t;
	t.reserve(n);
	for (size_t i = 0; i < n; ++i) {
		FbExtra* x = fbFind(fbs[i]);
		if (!x) { SRP_ERROR(FN, "Framebuffer %zu was not created by srpNewFramebuffer", i); return; }
		fbOtherWrite(x);
		t.push_back(FillTarget{ x->color, (uint32_t*) x->depth, x->stencil, fbs[i]->size });
	}
	if (!g.fillTargets.reserve(n * sizeof(FillTarget), FN)) return;
	g.rsDirty = true;
	/* from pageable memory: returns once the host vector has been read */
	if (!cudaOk(cudaMemcpyAsync(g.fillTargets.ptr, t.data(), n * sizeof(FillTarget), cudaMemcpyHostToDevice, g.stream),
	            FN, "cudaMemcpyAsync")) return;
	uint32_t dbits;
	memcpy(&dbits, &depth, 4);
	const unsigned ys = (unsigned) std::min<size_t>(n, 65535);
	k_fill_batch<<<dim3(16, ys), 256, 0, g.stream>>>(g.fillTargets.as<FillTarget>(), n, color, dbits, stencil, planes);
	++g.launches;
	if (g.fbMode == SRP_GPU_FB_COHERENT)
		for (size_t i = 0; i < n; ++i)
			for (size_t p = 0; p < fbs[i]->size; ++p) {
				if (planes & SRP_GPU_FILL_COLOR) fbs[i]->color[p] = color;
				if (planes & SRP_GPU_FILL_DEPTH) fbs[i]->depth[p] = depth;
				if (planes & SRP_GPU_FILL_STENCIL) fbs[i]->stencil[p] = stencil;
			}
}

void srpGpuFramebufferUpload(const SRPFramebuffer* fb)
{
	FbExtra* x = fbFind(fb);
	if (x) fbUpload(fb, x);
}

void srpGpuFramebufferFill(const SRPFramebuffer* fb, uint32_t color, float depth, uint8_t stencil, unsigned planes)
{
	FbExtra* x = fbFind(fb);
	if (!x) return;
	fbOtherWrite(x);
	g.rsDirty = true;
	uint32_t dbits;
	memcpy(&dbits, &depth, 4);
	if (planes & SRP_GPU_FILL_COLOR) fill32(x->color, color, fb->size);
	if (planes & SRP_GPU_FILL_DEPTH) fill32((uint32_t*) x->depth, dbits, fb->size);
	if (planes & SRP_GPU_FILL_STENCIL) cudaMemsetAsync(x->stencil, stencil, fb->size, g.stream);
	if (g.fbMode == SRP_GPU_FB_COHERENT) {
		for (size_t i = 0; i < fb->size; ++i) {
			if (planes & SRP_GPU_FILL_COLOR) fb->color[i] = color;
			if (planes & SRP_GPU_FILL_DEPTH) fb->depth[i] = depth;
			if (planes & SRP_GPU_FILL_STENCIL) fb->stencil[i] = stencil;
		}
	}
}

}  // extern "C"

/* ---------------------------------------------------------------- texture */

struct SRPTexture {
	uint8_t* rgb = nullptr;   /* host copy, 3 channels */
	int width = 0, height = 0, wm1 = 0, hm1 = 0;
	SRPTextureWrappingMode wx = TW_REPEAT, wy = TW_REPEAT;
	uint32_t* texels = nullptr;      /* device RGBA8: level 0, then the mip levels once built */
	TextureDesc* desc = nullptr;     /* device descriptor */
	bool dirty = true;
	/* filtering (srpTextureSetFilter): the mip chain, built on the host when
	 * TRILINEAR is first set, levels 1.. stored one after the other */
	SRPTextureFilter filter = SRP_TEXTURE_FILTER_NEAREST;
	int nLevels = 1;                 /* levels built */
	int lw[kMaxMipLevels] = {}, lh[kMaxMipLevels] = {};
	size_t loff[kMaxMipLevels] = {}; /* first texel of each level, level 0 included */
	std::vector<uint8_t> mips;       /* RGB8 of levels 1.. */
};

static const uint8_t* texelAt(const SRPTexture* t, int l, int x, int y)
{
	if (l == 0) return t->rgb + 3 * ((size_t) y * t->width + x);
	return t->mips.data() + 3 * (t->loff[l] - (size_t) t->width * t->height + (size_t) y * t->lw[l] + x);
}

/* The mip chain of srp/texture.h: level l + 1 is the 2x2 box average of
 * level l (edge texels repeated for odd sizes), rounded to nearest. */
static void textureBuildMips(SRPTexture* t)
{
	const int n = std::min(srpTextureMipLevels(t->width, t->height), kMaxMipLevels);
	t->lw[0] = t->width; t->lh[0] = t->height; t->loff[0] = 0;
	size_t at = (size_t) t->width * t->height;
	for (int l = 1; l < n; ++l) {
		t->lw[l] = std::max(1, t->lw[l - 1] / 2);
		t->lh[l] = std::max(1, t->lh[l - 1] / 2);
		t->loff[l] = at;
		at += (size_t) t->lw[l] * t->lh[l];
	}
	t->mips.assign((at - (size_t) t->width * t->height) * 3, 0);
	t->nLevels = n;
	for (int l = 1; l < n; ++l) {
		const int pw = t->lw[l - 1], ph = t->lh[l - 1];
		for (int j = 0; j < t->lh[l]; ++j)
			for (int i = 0; i < t->lw[l]; ++i) {
				const int x0 = std::min(2 * i, pw - 1), x1 = std::min(2 * i + 1, pw - 1);
				const int y0 = std::min(2 * j, ph - 1), y1 = std::min(2 * j + 1, ph - 1);
				const uint8_t *a = texelAt(t, l - 1, x0, y0), *b = texelAt(t, l - 1, x1, y0);
				const uint8_t *c = texelAt(t, l - 1, x0, y1), *d = texelAt(t, l - 1, x1, y1);
				uint8_t* o = (uint8_t*) texelAt(t, l, i, j);
				for (int k = 0; k < 3; ++k) o[k] = (uint8_t) ((a[k] + b[k] + c[k] + d[k] + 2) / 4);
			}
	}
}

/* Device texels of every level built so far (RGBA8), replacing the old copy. */
static bool textureUploadLevels(SRPTexture* t, const char* fn)
{
	const size_t n = t->loff[t->nLevels - 1] + (size_t) t->lw[t->nLevels - 1] * t->lh[t->nLevels - 1];
	std::vector<uint32_t> rgba(n);
	for (int l = 0; l < t->nLevels; ++l)
		for (int y = 0; y < t->lh[l]; ++y)
			for (int x = 0; x < t->lw[l]; ++x) {
				const uint8_t* p = texelAt(t, l, x, y);
				rgba[t->loff[l] + (size_t) y * t->lw[l] + x] = (uint32_t) p[0] | (uint32_t) p[1] << 8 | (uint32_t) p[2] << 16;
			}
	uint32_t* dev = nullptr;
	if (!cudaOk(cudaMalloc(&dev, n * 4), fn, "cudaMalloc")) return false;
	cudaMemcpy(dev, rgba.data(), n * 4, cudaMemcpyHostToDevice);
	if (t->texels) {
		/* draws queued with the old texels may still read them */
		cudaDeviceSynchronize();
		cudaFree(t->texels);
	}
	t->texels = dev;
	t->dirty = true;
	return true;
}

static bool textureSync(SRPTexture* t)
{
	if (!t->texels) {
		t->lw[0] = t->width; t->lh[0] = t->height; t->loff[0] = 0;
		if (!cudaOk(cudaMalloc(&t->desc, sizeof(TextureDesc)), "srpNewTexture", "cudaMalloc")) return false;
		if (!textureUploadLevels(t, "srpNewTexture")) return false;
	}
	if (t->dirty) {
		TextureDesc d = {};
		d.texels = t->texels;
		d.width = t->width; d.height = t->height; d.wm1 = t->wm1; d.hm1 = t->hm1;
		d.wrapX = t->wx; d.wrapY = t->wy;
		d.filter = t->filter;
		d.nLevels = t->filter == SRP_TEXTURE_FILTER_TRILINEAR ? t->nLevels : 1;
		for (int l = 0; l < t->nLevels; ++l) { d.lw[l] = t->lw[l]; d.lh[l] = t->lh[l]; d.loff[l] = (uint32_t) t->loff[l]; }
		cudaMemcpyAsync(t->desc, &d, sizeof d, cudaMemcpyHostToDevice, g.stream);
		cudaStreamSynchronize(g.stream);
		t->dirty = false;
	}
	return true;
}

/* Host bilinear sample of level l (channels in 0..255), as the device's. */
static void hostBilinear(const SRPTexture* t, int l, float u, float v, float c[3])
{
	const int w = t->lw[l], h = t->lh[l];
	const float x = (float) (w - 1) * u, y = (float) (h - 1) * (1.0f - v);
	const float fx0 = floorf(x), fy0 = floorf(y);
	const int x0 = std::min(std::max((int) fx0, 0), w - 1), y0 = std::min(std::max((int) fy0, 0), h - 1);
	const float fx = x - fx0, fy = y - fy0;
	const int x1 = x0 + 1 < w ? x0 + 1 : (t->wx == TW_REPEAT ? 0 : w - 1);
	const int y1 = y0 + 1 < h ? y0 + 1 : (t->wy == TW_REPEAT ? 0 : h - 1);
	const uint8_t *a = texelAt(t, l, x0, y0), *b = texelAt(t, l, x1, y0), *d = texelAt(t, l, x0, y1), *e = texelAt(t, l, x1, y1);
	for (int k = 0; k < 3; ++k) {
		const float top = (float) a[k] + fx * ((float) b[k] - (float) a[k]);
		const float bot = (float) d[k] + fx * ((float) e[k] - (float) d[k]);
		c[k] = top + fy * (bot - top);
	}
}

extern "C" {

SRPTexture* srpNewTextureFromMemory(const uint8_t* texels, int w, int h, int ch,
                                    SRPTextureWrappingMode wx, SRPTextureWrappingMode wy)
{
	if (!texels || w <= 0 || h <= 0 || (ch != 3 && ch != 4)) {
		SRP_ERROR("srpNewTextureFromMemory", "Invalid texture arguments");
		return nullptr;
	}
	if (!ensureInit("srpNewTextureFromMemory")) return nullptr;
	SRPTexture* t = new SRPTexture();
	t->rgb = (uint8_t*) malloc((size_t) w * h * 3);
	for (size_t i = 0; i < (size_t) w * h; ++i) memcpy(t->rgb + 3 * i, texels + (size_t) ch * i, 3);
	t->width = w; t->height = h; t->wm1 = w - 1; t->hm1 = h - 1; t->wx = wx; t->wy = wy;
	if (!textureSync(t)) { free(t->rgb); delete t; return nullptr; }
	return t;
}

SRPTexture* srpNewTexture(const char* path, SRPTextureWrappingMode wx, SRPTextureWrappingMode wy)
{
	SRPImage img;
	const char* err = "";
	if (!srpImageLoad(path, &img, &err)) {
		SRP_ERROR("srpNewTexture", "Failed to load image `%s`: %s", path, err);
		return nullptr;
	}
	SRPTexture* t = srpNewTextureFromMemory(img.rgb, img.width, img.height, 3, wx, wy);
	free(img.rgb);
	return t;
}

void srpFreeTexture(SRPTexture* t)
{
	if (!t) return;
	cudaStreamSynchronize(g.stream);
	if (t->texels) cudaFree(t->texels);
	if (t->desc) cudaFree(t->desc);
	free(t->rgb);
	delete t;
}

int srpTextureMipLevels(int w, int h)
{
	int n = 1;
	while (w > 1 || h > 1) { w = w > 1 ? w / 2 : 1; h = h > 1 ? h / 2 : 1; ++n; }
	return n;
}

void srpTextureSetFilter(SRPTexture* t, SRPTextureFilter f)
{
	if (!t) return;
	if (f != SRP_TEXTURE_FILTER_NEAREST && f != SRP_TEXTURE_FILTER_BILINEAR && f != SRP_TEXTURE_FILTER_TRILINEAR) {
		SRP_ERROR("srpTextureSetFilter", "Unknown texture filter (%i). Falling back to SRP_TEXTURE_FILTER_NEAREST", (int) f);
		f = SRP_TEXTURE_FILTER_NEAREST;
	}
	if (f == SRP_TEXTURE_FILTER_TRILINEAR && t->nLevels == 1 && srpTextureMipLevels(t->width, t->height) > 1) {
		/* the chain is built once, here: draws then allocate nothing for it */
		textureBuildMips(t);
		if (!textureUploadLevels(t, "srpTextureSetFilter")) return;
	}
	t->filter = f;
	t->dirty = true;
}

SRPTextureFilter srpTextureGetFilter(const SRPTexture* t) { return t ? t->filter : SRP_TEXTURE_FILTER_NEAREST; }

void srpTextureGetFilteredColorLod(const SRPTexture* t, float u, float v, float lod, float out[4])
{
	if (t->filter == SRP_TEXTURE_FILTER_NEAREST) { srpTextureGetFilteredColor(t, u, v, out); return; }
	if (u < 0 || u > 1) u = (float) (t->wx == TW_REPEAT ? (double) u - floor(u) : fmax(0.0, fmin(1.0, u)));
	if (v < 0 || v > 1) v = (float) (t->wy == TW_REPEAT ? (double) v - floor(v) : fmax(0.0, fmin(1.0, v)));
	float c[3];
	hostBilinear(t, 0, u, v, c);
	if (t->filter == SRP_TEXTURE_FILTER_TRILINEAR && t->nLevels > 1) {
		const float top = (float) (t->nLevels - 1);
		const float ld = lod > 0.0f ? (lod < top ? lod : top) : 0.0f;
		const int l0 = (int) floorf(ld);
		const float f = ld - (float) l0;
		float c0[3], c1[3];
		hostBilinear(t, l0, u, v, c0);
		hostBilinear(t, l0 + 1 < t->nLevels ? l0 + 1 : l0, u, v, c1);
		for (int k = 0; k < 3; ++k) c[k] = c0[k] + f * (c1[k] - c0[k]);
	}
	const float inv255 = (float) (1. / 255.);
	for (int k = 0; k < 3; ++k) out[k] = c[k] * inv255;
	out[3] = 1.f;
}

void srpTextureGetFilteredColor(const SRPTexture* t, float u, float v, float out[4])
{
	/* host lookup, same arithmetic as the device sampler (texture.c:56-81) */
	if (t->filter != SRP_TEXTURE_FILTER_NEAREST) { srpTextureGetFilteredColorLod(t, u, v, 0.0f, out); return; }
	if (u < 0 || u > 1) u = (float) (t->wx == TW_REPEAT ? (double) u - floor(u) : fmax(0.0, fmin(1.0, u)));
	if (v < 0 || v > 1) v = (float) (t->wy == TW_REPEAT ? (double) v - floor(v) : fmax(0.0, fmin(1.0, v)));
	float x = (float) t->wm1 * u;
	float y = (float) t->hm1 * (1 - v);
	size_t xi = (size_t) ((double) x + 0.5), yi = (size_t) ((double) y + 0.5);
	const uint8_t* p = t->rgb + 3 * (xi + yi * (size_t) t->width);
	const float inv255 = (float) (1. / 255.);
	out[0] = p[0] * inv255; out[1] = p[1] * inv255; out[2] = p[2] * inv255; out[3] = 1.f;
}

int srpTextureGet(SRPTexture* t, SRPTextureParameter p)
{
	switch (p) {
	case SRP_TEXTURE_WRAPPING_MODE_X: return t->wx;
	case SRP_TEXTURE_WRAPPING_MODE_Y: return t->wy;
	}
	SRP_ERROR("srpTextureGet", "Unknown texture parameter (%i)", (int) p);
	return -1;
}

void srpTextureSet(SRPTexture* t, SRPTextureParameter p, int data)
{
	if (p != SRP_TEXTURE_WRAPPING_MODE_X && p != SRP_TEXTURE_WRAPPING_MODE_Y) {
		SRP_ERROR("srpTextureSet", "Unknown texture parameter (%i)", (int) p);
		return;
	}
	if (p == SRP_TEXTURE_WRAPPING_MODE_X) t->wx = (SRPTextureWrappingMode) data;
	else t->wy = (SRPTextureWrappingMode) data;
	t->dirty = true;
	if (data != TW_REPEAT && data != TW_CLAMP_TO_EDGE)
		SRP_ERROR("srpTextureSet", "Unknown texture wrapping mode (%i). Falling back to TW_REPEAT", data);
}

/* ---------------------------------------------------------------- shaders */

void srpGpuRegisterVertexShader(void (*fn)(SRPVertexShaderIn*, SRPVertexShaderOut*), SRPGpuVertexShaderId id)
{
	for (auto& e : g.reg.vs) if (e.first == (void*) fn) { e.second = id; return; }
	g.reg.vs.push_back({ (void*) fn, (int) id });
}

void srpGpuRegisterFragmentShader(void (*fn)(SRPFragmentShaderIn*, SRPFragmentShaderOut*), SRPGpuFragmentShaderId id)
{
	for (auto& e : g.reg.fs) if (e.first == (void*) fn) { e.second = id; return; }
	g.reg.fs.push_back({ (void*) fn, (int) id });
}

}  // extern "C"

/* the library's own host copies of the shared shaders */
#define SRP_SHADERLIB_HOST_ONLY
extern "C" {
#include "srp/shaderlib_host.inc"
}

static int lookupVS(void* fn)
{
	if (fn == (void*) srpVsTransform) return SRP_GPU_VS_TRANSFORM;
	if (fn == (void*) srpVsWorld) return SRP_GPU_VS_WORLD;
	if (fn == (void*) srpVsBytes) return SRP_GPU_VS_BYTES;
	for (auto& e : g.reg.vs) if (e.first == fn) return e.second;
	return 0;
}

static int lookupFS(void* fn)
{
	static const struct { void* f; int id; } builtin[] = {
		{ (void*) srpFsVaryingColor, SRP_GPU_FS_VARYING_COLOR }, { (void*) srpFsSolid, SRP_GPU_FS_SOLID },
		{ (void*) srpFsPrimitiveId, SRP_GPU_FS_PRIMITIVE_ID }, { (void*) srpFsTexture, SRP_GPU_FS_TEXTURE },
		{ (void*) srpFsTextureModulate, SRP_GPU_FS_TEXTURE_MODULATE }, { (void*) srpFsBlinnPhong, SRP_GPU_FS_BLINN_PHONG },
		{ (void*) srpFsMarble, SRP_GPU_FS_MARBLE }, { (void*) srpFsDepthOverwrite, SRP_GPU_FS_DEPTH_OVERWRITE },
		{ (void*) srpFsFragCoord, SRP_GPU_FS_FRAGCOORD }, { (void*) srpFsFlatInt, SRP_GPU_FS_FLAT_INT },
		{ (void*) srpFsMixed, SRP_GPU_FS_MIXED }, { (void*) srpFsBytePalette, SRP_GPU_FS_BYTE_PALETTE },
		{ (void*) srpFsPrimitiveMod, SRP_GPU_FS_PRIMITIVE_MOD }, { (void*) srpFsTextureLod, SRP_GPU_FS_TEXTURE_LOD },
	};
	for (auto& b : builtin) if (b.f == fn) return b.id;
	for (auto& e : g.reg.fs) if (e.first == fn) return e.second;
	return 0;
}

/* ------------------------------------------------------------------- draw */

static size_t varyingElemSize(SRPType t)
{
	switch (t) {
	case SRP_INT8: case SRP_UINT8: return 1;
	case SRP_INT16: case SRP_UINT16: return 2;
	case SRP_INT32: case SRP_UINT32: case SRP_FLOAT: return 4;
	case SRP_INT64: case SRP_UINT64: case SRP_DOUBLE: return 8;
	}
	return 0;
}

static bool buildLayout(const SRPVertexShader* vs, VaryingLayout& L)
{
	memset(&L, 0, sizeof L);
	if (vs->nVaryings > (size_t) kMaxVaryings) {
		SRP_ERROR("srpDraw", "GPU path supports at most %d varyings (got %zu)", kMaxVaryings, vs->nVaryings);
		return false;
	}
	size_t off = 0;
	bool floatOnly = true;
	for (size_t a = 0; a < vs->nVaryings; ++a) {
		const SRPVaryingInfo& in = vs->varyingsInfo[a];
		const size_t es = varyingElemSize(in.type);
		if (!es) SRP_ERROR("interpolateAttributes", "Unexpected type (%i)", (int) in.type);
		VaryingAttr& at = L.attr[a];
		at.offset = (uint16_t) off;
		at.nItems = (uint16_t) in.nItems;
		at.type = (uint8_t) in.type;
		at.mode = (uint8_t) (in.interpolationMode == SRP_INTERPOLATION_MODE_PERSPECTIVE ? kPerspective
		                   : in.interpolationMode == SRP_INTERPOLATION_MODE_AFFINE ? kAffine : kFlat);
		at.elemSize = (uint8_t) es;
		if (es != 4 || (off & 3)) floatOnly = false;
		for (size_t e = 0; e < in.nItems && es == 4 && !(off & 3); ++e) {
			const size_t w = off / 4 + e;
			if (w < (size_t) kMaxVaryingWords) {
				L.wordMode[w] = at.mode;
				L.wordIsFloat[w] = in.type == SRP_FLOAT;
			}
		}
		off += es * in.nItems;
	}
	const size_t bytes = std::max(off, vs->varyingsSize);
	if (bytes > (size_t) 4 * kMaxVaryingWords) {
		SRP_ERROR("srpDraw", "GPU path supports varying blocks up to %d bytes (got %zu)", 4 * kMaxVaryingWords, bytes);
		return false;
	}
	L.nAttr = (int) vs->nVaryings;
	L.sizeBytes = (int) bytes;
	L.nWords = (int) ((bytes + 3) / 4);
	/* words outside any attribute are copied from the provoking vertex */
	for (int w = (int) ((off + 3) / 4); w < L.nWords; ++w) { L.wordMode[w] = kFlat; L.wordIsFloat[w] = 0; }
	L.floatOnly = floatOnly ? 1 : 0;
	return true;
}

static bool isTri(SRPPrimitive p) { return p == SRP_PRIM_TRIANGLES || p == SRP_PRIM_TRIANGLE_STRIP || p == SRP_PRIM_TRIANGLE_FAN; }
static bool isLine(SRPPrimitive p) { return p == SRP_PRIM_LINES || p == SRP_PRIM_LINE_STRIP || p == SRP_PRIM_LINE_LOOP; }

static bool uploadVB(SRPVertexBuffer* vb)
{
	if (!vb->dirty && vb->dev.ptr) return true;
	if (!vb->dev.reserve(vb->nBytes + 16, "srpDraw")) return false;
	if (vb->nBytes) cudaMemcpyAsync(vb->dev.ptr, vb->host, vb->nBytes, cudaMemcpyHostToDevice, copyStreamReady());
	vb->dirty = false;
	markUpload(vb->ready, vb->readyOwned, vb->pending, vb->seq);
	return true;
}

static bool uploadIB(SRPIndexBuffer* ib)
{
	if (!ib->dirty && ib->dev.ptr) return true;
	if (!ib->dev.reserve(ib->nBytes + 16, "srpDraw")) return false;
	if (ib->nBytes) cudaMemcpyAsync(ib->dev.ptr, ib->host, ib->nBytes, cudaMemcpyHostToDevice, copyStreamReady());
	ib->dirty = false;
	markUpload(ib->ready, ib->readyOwned, ib->pending, ib->seq);
	return true;
}

/* Copies both sets' counters to their host mirrors (waits for the GPU) and
 * returns the fragments counted by all draws. */
static unsigned long long readCounters()
{
	syncFronts();
	cudaStreamSynchronize(g.resolveStream);
	for (DrawSet& S : g.sets)
		cudaMemcpyAsync(S.hostCtr, S.ctr.ptr, sizeof(DeviceCounters), cudaMemcpyDeviceToHost, g.stream);
	if (!cudaOk(cudaStreamSynchronize(g.stream), "srpDraw", "kernel execution")) return 0;
	return g.sets[0].hostCtr->fragments + g.sets[1].hostCtr->fragments;
}

/* Room for the clip pre-pass's fans of filled triangles: g.clipPolyCap
 * slots of kClipFan records each. */
static bool reserveClipFans(DrawSet& S, const char* fn)
{
	const size_t slots = g.clipPolyCap;
	return S.clipFan.reserve(slots * sizeof(uint2), fn) && S.clipR.reserve(slots * kClipFan * sizeof(TriRaster), fn) &&
	       S.clipA.reserve(slots * kClipFan * sizeof(TriAttr), fn);
}

static void setClipFans(DrawParams& P, DrawSet& S)
{
	P.clipFan = S.clipFan.as<uint2>();
	P.clipR = S.clipR.as<TriRaster>();
	P.clipA = S.clipA.as<TriAttr>();
}

/* The GPU pipeline for one draw call. */
static void runDraw(const SRPIndexBuffer* ibc, const SRPVertexBuffer* vbc, const SRPFramebuffer* fb,
                    const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count, size_t nIn)
{
	const char* FN = "srpDraw";
	SRPIndexBuffer* ib = (SRPIndexBuffer*) ibc;
	SRPVertexBuffer* vb = (SRPVertexBuffer*) vbc;
	FbExtra* fx = fbFind(fb);
	if (!fx) { SRP_ERROR(FN, "Framebuffer was not created by srpNewFramebuffer"); return; }
	/* after its download in flight; until the draw has been queued in full,
	 * downloads of this framebuffer go back to the library's stream */
	fbAfterDownloads(fx);
	fx->lastWrite = nullptr;
	const int vsId = lookupVS((void*) sp->vs->shader);
	const int fsId = lookupFS((void*) sp->fs->shader);
	if (!vsId || !fsId) {
		SRP_ERROR(FN, "Shader has no GPU implementation; map it with srpGpuRegisterVertexShader/FragmentShader");
		return;
	}
	if (vb->stride == 0 || vb->stride > 1024) {
		SRP_ERROR(FN, "GPU path supports vertex strides of 1..1024 bytes (got %zu)", vb->stride);
		return;
	}
	static DrawParams P;
	memset(&P, 0, sizeof P);
	if (!buildLayout(sp->vs, P.L)) return;
	if (g.tuneArmed) { cudaEventRecord(g.tuneStart, g.stream); g.tuneArmed = false; }
	/* this draw's scratch set and front stream */
	DrawSet& S = g.sets[g.setNext];
	g.setNext ^= 1;
	const cudaStream_t fs = (g.overlap && !g.profiling) ? S.front : g.stream;
	/* state snapshot */
	DrawState& st = P.st;
	st.W = (int) fb->width; st.H = (int) fb->height;
	st.frontFaceCW = srpContext.raster.frontFace == SRP_WINDING_CW;
	st.cullFace = srpContext.raster.cullFace;
	st.polygonMode = srpContext.raster.polygonMode;
	st.pointSize = srpContext.raster.pointSize;
	st.provokingFirst = srpContext.provokingVertexMode == SRP_PROVOKING_VERTEX_FIRST;
	st.scissorEnabled = srpContext.scissor.enabled;
	st.sx0 = srpContext.scissor.x; st.sx1 = srpContext.scissor.x + srpContext.scissor.width;
	st.sy0 = srpContext.scissor.y; st.sy1 = srpContext.scissor.y + srpContext.scissor.height;
	st.stencilEnabled = srpContext.stencil.enabled;
	const SRPStencilFaceState* fsrc[2] = { &srpContext.stencil.front, &srpContext.stencil.back };
	StencilFace* fdst[2] = { &st.front, &st.back };
	for (int i = 0; i < 2; ++i) {
		fdst[i]->func = fsrc[i]->func; fdst[i]->sfail = fsrc[i]->sfailOp; fdst[i]->dfail = fsrc[i]->dfailOp;
		fdst[i]->pass = fsrc[i]->passOp; fdst[i]->ref = fsrc[i]->ref; fdst[i]->mask = fsrc[i]->mask;
		fdst[i]->writeMask = fsrc[i]->writeMask;
	}
	st.depthTest = srpContext.depth.testEnable;
	st.depthWrite = srpContext.depth.writeEnable;
	st.depthOp = srpContext.depth.compareOp;
	st.earlyZ = !sp->fs->mayOverwriteDepth;
	st.tile = kTile;
	st.tilesX = (st.W + kTile - 1) / kTile;
	st.tilesY = (st.H + kTile - 1) / kTile;
	const uint32_t numTiles = (uint32_t) st.tilesX * (uint32_t) st.tilesY;
	/* uniform: the built-in shaders read SRPStdUniform; its texture pointer
	 * is replaced by the texture's device descriptor */
	if (sp->uniform) {
		SRPStdUniform u;
		memcpy(&u, sp->uniform, sizeof u);
		if (u.texture) {
			SRPTexture* t = u.texture;
			if (!textureSync(t)) return;
			u.texture = (SRPTexture*) t->desc;
		}
		memcpy(P.uniform, &u, sizeof u);
	}
	static_assert(sizeof(SRPStdUniform) <= kMaxUniformBytes, "uniform too large");
	P.vsId = vsId;
	P.fsId = fsId;
	P.heavyItems = g.tune.heavyItems;
	P.spinLimit = g.spinLimit;
	P.waitTest = g.waitTest;
	P.heavyCtasPerSM = g.tune.heavyCtasPerSM;
	P.prim = prim;
	P.start = start;
	P.count = count;
	P.nIn = (int) nIn;
	if (!uploadVB(vb)) return;
	P.vertices = vb->dev.as<unsigned char>();
	P.nVertices = vb->nVertices;
	P.stride = (int) vb->stride;
	if (ib) {
		if (!uploadIB(ib)) return;
		P.indices = ib->dev.ptr;
		P.indexSize = (int) ib->elemSize;
		/* as many indices as vertices: the range very likely covers the
		 * buffer, so every vertex is shaded (the shader is a pure function;
		 * unreferenced results are never read) and the range pass is skipped */
		P.shadeAll = count >= vb->nVertices ? 1 : 0;
		if (ib->type != SRP_UINT8 && ib->type != SRP_UINT16 && ib->type != SRP_UINT32 && ib->type != SRP_UINT64) {
			SRP_ERROR("indexIndexBuffer", "Unexpected type (%i)", (int) ib->type);
			return;
		}
	}
	P.minmax = S.minmax.as<unsigned long long>();
	P.ctr = S.ctr.as<DeviceCounters>();
	P.color = fx->color;
	P.depth = fx->depth;
	P.stencil = fx->stencil;
	const int mode = isTri(prim) ? st.polygonMode : (isLine(prim) ? SRP_POLYGON_MODE_LINE : SRP_POLYGON_MODE_POINT);
	const int kind = mode == SRP_POLYGON_MODE_FILL ? kKindTri : mode == SRP_POLYGON_MODE_LINE ? kKindLineFrag : kKindPoint;
	const size_t outPer = isTri(prim) && mode != SRP_POLYGON_MODE_FILL ? 3 : 1;
	if (g.fbMode == SRP_GPU_FB_COHERENT) fbUpload(fb, fx);

	uint32_t primCap = (uint32_t) std::min<size_t>(nIn * outPer + 4096, 0x3FFFFFFFu);
	uint32_t entryCap = (uint32_t) std::min<double>((double) (nIn * outPer) * g.entryRatio[kind] + 4096, 4.0e9);
	if (kind == kKindLineFrag) entryCap = std::min(entryCap, kMaxLineEntries);
	const uint32_t keyBits = sortKeyBits(numTiles);
	const bool late = sp->fs->mayOverwriteDepth && shadeSupportsLateDepth(fsId);
	const bool learned = learnedPrepare(P, kind, late, 1, g.stream);
	/* the resolve runs beside the previous draw's shading, except for
	 * late-depth draws, whose resolve writes colour */
	const cudaStream_t rs = fs != g.stream && !late ? g.resolveStream : g.stream;
	bool drawn = false;
	for (int attempt = 0; attempt < 4 && !drawn; ++attempt) {
		/* long lines are queued in the big-job buffer: room for every line */
		if (kind == kKindLineFrag && g.bigCap < primCap) g.bigCap = primCap;
		const uint32_t rows = (uint32_t) vb->nVertices + g.clipRows;
		const size_t nw = (size_t) std::max(P.L.nWords, 1);
		const uint32_t blocks = (uint32_t) ((nIn + kSetupThreads - 1) / kSetupThreads);
		bool ok = S.clip.reserve((size_t) rows * 16, FN) && S.vary.reserve((size_t) rows * nw * 4, FN) &&
		          S.vset0.reserve((size_t) vb->nVertices * 16 + 16, FN) && S.vset1.reserve((size_t) vb->nVertices * 16 + 16, FN) &&
		          S.codes.reserve((size_t) vb->nVertices + 16, FN) &&
		          S.lookback.reserve((size_t) std::max(blocks, 1u) * 8, FN) &&
		          S.keys.reserve((size_t) entryCap * 4, FN) && S.vals.reserve((size_t) entryCap * 4, FN) &&
		          S.keys2.reserve((size_t) entryCap * 4, FN) && S.vals2.reserve((size_t) entryCap * 4, FN) &&
		          S.hist.reserve(sortHistWords(entryCap) * 4, FN) && S.partials.reserve(sortPartialWords(entryCap) * 4 + 64, FN) &&
		          S.big.reserve((size_t) g.bigCap * 16, FN) && S.table.reserve((size_t) g.tableCap * 4, FN) &&
		          S.clipSlot.reserve((size_t) nIn * 4 + 4, FN) &&
		          S.clipPolys.reserve((size_t) g.clipPolyCap * (1 + kMaxPoly) * 4, FN) &&
		          S.tileStart.reserve((size_t) (numTiles + 1) * 4, FN) && S.tileEnd.reserve((size_t) (numTiles + 1) * 4, FN) &&
		          S.winner.reserve(fb->size * 4 + 4, FN) && S.heavy.reserve((size_t) (numTiles + 1) * 4, FN);
		if (kind == kKindTri) ok = ok && S.triR.reserve((size_t) primCap * sizeof(TriRaster), FN) &&
		                           S.triA.reserve((size_t) primCap * sizeof(TriAttr), FN) &&
		                           reserveClipFans(S, FN);
		else if (kind == kKindPoint) ok = ok && S.points.reserve((size_t) primCap * sizeof(PointRec), FN);
		else ok = ok && S.lines.reserve((size_t) primCap * sizeof(LineRec), FN) &&
		          S.frags.reserve((size_t) entryCap * kRunFrags * sizeof(LineFrag), FN) &&
		          S.fragVals.reserve((size_t) entryCap * kRunFrags * 4, FN) &&
		          S.runSums.reserve((size_t) runSumWords(entryCap) * 4, FN);
		if (!ok) return;
		P.clip = S.clip.as<float4>();
		P.vset0 = S.vset0.as<float4>();
		P.vset1 = S.vset1.as<float4>();
		P.codes = S.codes.as<uint8_t>();
		P.vary = S.vary.as<uint32_t>();
		P.clipBase = (uint32_t) vb->nVertices;
		P.clipCap = g.clipRows;
		P.triR = S.triR.as<TriRaster>();
		P.triA = S.triA.as<TriAttr>();
		P.lines = S.lines.as<LineRec>();
		P.points = S.points.as<PointRec>();
		P.frags = S.frags.as<LineFrag>();
		P.primCap = primCap;
		P.fragCap = kind == kKindLineFrag ? (unsigned long long) entryCap * kRunFrags : 0;
		P.fragVals = S.fragVals.as<uint32_t>();
		P.runSums = S.runSums.as<uint32_t>();
		P.keys = S.keys.as<uint32_t>();
		P.vals = S.vals.as<uint32_t>();
		P.entryCap = entryCap;
		P.bigJobs = S.big.as<uint4>();
		P.bigCap = g.bigCap;
		P.table = S.table.as<float>();
		P.clipSlot = S.clipSlot.as<uint32_t>();
		P.clipPolys = S.clipPolys.as<uint32_t>();
		P.clipPolyCap = g.clipPolyCap;
		setClipFans(P, S);
		P.tableCap = g.tableCap;
		P.lookback = S.lookback.as<unsigned long long>();
		P.tileStart = S.tileStart.as<uint32_t>();
		P.tileEnd = S.tileEnd.as<uint32_t>();
		P.winner = S.winner.as<int32_t>();
		/* framebuffer tiles by TMA where the planes allow it */
		P.tma = g.tma && encodeTileMap(&P.tmDepth, P.depth, st.W, st.H, CU_TENSOR_MAP_DATA_TYPE_FLOAT32) &&
		        encodeTileMap(&P.tmWinner, P.winner, st.W, st.H, CU_TENSOR_MAP_DATA_TYPE_INT32) &&
		        encodeTileMap(&P.tmColor, P.color, st.W, st.H, CU_TENSOR_MAP_DATA_TYPE_UINT32) ? g.tma : 0u;

		/* the whole draw is enqueued before the host looks at any count */
		uint32_t* sk = nullptr;
		uint32_t* sv = nullptr;
		auto head = [&]() {
			stageBegin();
			launchReset(P, fs);
			if (ib && !P.shadeAll) launchIndexRange(P, fs);
			if (ib) launchVertex(P, 0, vb->nVertices, fs);
			else launchVertex(P, start, count, fs);
			stageEnd(SRP_GPU_STAGE_VERTEX, ib && !P.shadeAll ? 3 : 2);
		};
		auto head2 = [&]() {
			stageBegin();
			cudaMemsetAsync(P.lookback, 0, (size_t) blocks * 8, fs);
			if (isTri(prim)) launchClipPrepass(P, fs);
			launchSetup(P, fs);
			launchCheck(P, fs);
			stageEnd(SRP_GPU_STAGE_SETUP, isTri(prim) ? 3 : 2);
		};
		/* lambda tables (triangles only): needed by the resolve, not by the
		 * binning, so they run on the resolve stream beside the bin */
		auto mid = [&]() {
			stageBegin();
			launchLambdaTables(P, g.bigJobsSeen[kind], rs);
			stageEnd(SRP_GPU_STAGE_BIN, 1);
		};
		auto bin = [&]() {
			stageBegin();
			if (kind == kKindLineFrag) launchLineFrags(P, fs);
			else launchBigEntries(P, g.bigJobsSeen[kind], fs);
			sortEntries(P, keyBits, S.keys2.as<uint32_t>(), S.vals2.as<uint32_t>(), S.hist.as<uint32_t>(),
			            S.partials.as<uint32_t>(), &sk, &sv, fs);
			cudaMemsetAsync(P.tileStart, 0, (size_t) numTiles * 4, fs);
			cudaMemsetAsync(P.tileEnd, 0, (size_t) numTiles * 4, fs);
			if (kind == kKindLineFrag) {
				/* the sorted runs back to fragments: the resolve takes one item per fragment */
				launchRunExpand(P, sk, sv, numTiles, fs);
				sv = P.fragVals;
			} else {
				launchTileRanges(P, sk, numTiles, fs);
			}
			stageEnd(SRP_GPU_STAGE_BIN, 2 + 1 + (int) (keyBits / 8) + 1 + (kind == kKindLineFrag ? 2 : 0));
		};
		auto resolve = [&]() {
			stageBegin();
			if (late) launchResolveLate(P, kind, sv, numTiles, rs);
			else launchResolve(P, kind, sv, numTiles, S.heavy.as<uint32_t>(), rs, g.auxStream, g.forkEvent, g.joinEvent);
			stageEnd(SRP_GPU_STAGE_RESOLVE, late ? 1 : 3);
		};
		auto shade = [&]() {
			stageBegin();
			launchShade(P, kind, numTiles, g.stream);
			stageEnd(SRP_GPU_STAGE_SHADE, 1);
		};
		/* the front waits for the last draw that used this set (on the
		 * library's stream) and for the uploads of the buffers it reads (on
		 * the copy stream); when the whole vertex buffer is shaded, the vertex
		 * stage needs no indices and the index upload is waited for before
		 * setup only */
		const bool lateIb = ib && P.shadeAll && ib->ready;
		if (fs != g.stream) cudaStreamWaitEvent(fs, S.rasterDone, 0);
		if (vb->ready) cudaStreamWaitEvent(fs, vb->ready, 0);
		if (ib && ib->ready && !lateIb) cudaStreamWaitEvent(fs, ib->ready, 0);
		runDrawSeq(graphKey(P, { (unsigned long long) kind, late, ib != nullptr, start, count, vb->nVertices, blocks,
		                         keyBits, numTiles, g.bigJobsSeen[kind], (unsigned long long) (uintptr_t) g.stream,
		                         (unsigned long long) (uintptr_t) fs, (unsigned long long) (uintptr_t) rs }),
		           S, fs, rs, head, lateIb ? ib->ready : nullptr, head2, kind == kKindTri, mid, bin, resolve, !late, shade);
		g.launches += 4 + (ib && !P.shadeAll ? 1 : 0) + (isTri(prim) ? 1 : 0) + (kind == kKindPoint ? 1 : 2) + 1 +
		              keyBits / 8 + 1 + (kind == kKindLineFrag ? 2 : 0) +
		              (late ? 1 : 4);
		if (!cudaOk(cudaGetLastError(), FN, "launch")) return;
		/* wait for the setup counters only; the rest of the draw runs on */
		if (!cudaOk(cudaEventSynchronize(S.ctrEvent), FN, "kernel execution")) return;
		const DeviceCounters c = *S.hostCtr;
		if (c.errors & kErrBadIndex) {
			SRP_ERROR(FN, "Vertex index out of range of the vertex buffer (%zu vertices)", vb->nVertices);
			return;
		}
		if (c.errors & kErrSpin) { SRP_ERROR(FN, "Ordered-compaction wait timed out"); return; }
		if (c.abort) {
			/* the enqueued rest of the draw skipped itself; grow and draw again */
			cudaStreamSynchronize(fs);
			cudaStreamSynchronize(g.stream);
			bool grew = false;
			if (c.clipVerts > g.clipRows) { g.clipRows = (uint32_t) std::min<unsigned long long>(c.clipVerts * 2, 0x7FFFFFFF); grew = true; }
			if (c.prims > primCap) { primCap = (uint32_t) std::min<unsigned long long>(c.prims + 1024, 0x3FFFFFFF); grew = true; }
			if (c.entries > entryCap) {
				const double cap = kind == kKindLineFrag ? (double) kMaxLineEntries : 4.0e9;
				const uint32_t want = (uint32_t) std::min<double>(c.entries * 1.25 + 1024, cap);
				if (want > entryCap) { entryCap = want; grew = true; }
			}
			if (c.bigJobs > g.bigCap) { g.bigCap = (uint32_t) std::min<unsigned long long>(c.bigJobs * 2, 1u << 30); grew = true; }
			if (c.clipTris > g.clipPolyCap) { g.clipPolyCap = (uint32_t) std::min<unsigned long long>(c.clipTris * 2, 1u << 30); grew = true; }
			if (c.tableWords > g.tableCap) { g.tableCap = std::min<unsigned long long>(c.tableWords * 5 / 4 + 1024, 0xFFFFFFFFull); grew = true; }
			if (!grew) { SRP_ERROR(FN, "Scratch capacity exceeded"); return; }
			++g.stats.drawRetries;
			continue;
		}
		g.entryRatio[kind] = std::max(0.25, std::min(4096.0, (double) c.entries / (double) (nIn * outPer) * 1.25));
		g.bigJobsSeen[kind] = (uint32_t) std::min<unsigned long long>(c.bigJobs, 1u << 30);
		g.stats.primitives += c.prims;
		g.stats.binEntries += c.entries;
		g.stats.clipOverflows += c.clipOverflow;
		g.profile.resolveTiles += numTiles;
		g.profile.resolveItems += c.entries;
		drawn = true;
	}
	if (!drawn) { SRP_ERROR(FN, "Scratch capacity could not be sized for the draw"); return; }
	if (learned) {
		/* the judge found the network too far from the shader: shade again */
		uint8_t redo = 0;
		if (learnedJudge(1, &redo, nullptr, g.stream, P.ctr)) {
			P.fsId = P.judgeFs;
			stageBegin();
			launchShade(P, kind, numTiles, g.stream);
			stageEnd(SRP_GPU_STAGE_SHADE, 1);
			++g.launches;
			if (fs != g.stream) cudaEventRecord(S.rasterDone, g.stream);
		}
	}
	++g.stats.draws;
	fx->lastWrite = drawWriteEvent(fx->lastWriteSeq);
	if (g.fbMode == SRP_GPU_FB_COHERENT) fbDownload(fb, fx);
}

static void warnExcess(SRPPrimitive p, size_t n)
{
	if (p == SRP_PRIM_LINES && n % 2 != 0)
		message(SRP_MESSAGE_WARNING, SRP_MESSAGE_SEVERITY_LOW, "warnOnExcessVertexCount",
		        "Odd vertex count when drawing SRP_PRIM_LINES. The last vertex will be ignored\n");
	if (p == SRP_PRIM_TRIANGLES && n % 3 != 0)
		message(SRP_MESSAGE_WARNING, SRP_MESSAGE_SEVERITY_LOW, "warnOnExcessVertexCount",
		        "Vertex count not divisible by 3 when drawing SRP_PRIM_TRIANGLES. The last %i vertex/vertices will be ignored\n",
		        (int) (n % 3));
}

/* drawBuffer (src/pipeline/draw.c:63-82): range check, primitive class,
 * early returns, then the GPU pipeline. */
static void drawBuffer(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                       const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count)
{
	if (count == 0) return;
	const size_t end = start + count - 1;
	const size_t size = ib ? ib->nIndices : vb->nVertices;
	if (end >= size) {
		SRP_ERROR("checkOOB", ib ? "Attempt to OOB access index buffer (read) at indices %zu-%zu (size: %zu)\n"
		                         : "Attempt to OOB access vertex buffer (read) at indices %zu-%zu (size: %zu)\n",
		          start, end, size);
		return;
	}
	size_t nIn = 0;
	if (isTri(prim)) {
		if (srpContext.raster.cullFace == SRP_FACE_FRONT_AND_BACK) return;
		warnExcess(prim, count);
		nIn = prim == SRP_PRIM_TRIANGLES ? count / 3 : (count >= 3 ? count - 2 : 0);
		if (srpContext.raster.polygonMode != SRP_POLYGON_MODE_FILL && srpContext.raster.polygonMode != SRP_POLYGON_MODE_LINE &&
		    srpContext.raster.polygonMode != SRP_POLYGON_MODE_POINT) {
			SRP_ERROR("assembleTrianglesGeneric", "Unexpected srpContext.raster.polygonMode (%i)", (int) srpContext.raster.polygonMode);
			return;
		}
	} else if (isLine(prim)) {
		warnExcess(prim, count);
		nIn = prim == SRP_PRIM_LINES ? count / 2 : (count != 1 ? (prim == SRP_PRIM_LINE_STRIP ? count - 1 : count) : 0);
	} else if (prim == SRP_PRIM_POINTS) {
		if (srpContext.raster.pointSize <= 0.) return;
		nIn = count;
	} else {
		SRP_ERROR("drawBuffer", "Unknown primitive type: %i", (int) prim);
		return;
	}
	if (nIn == 0) return;
	if (nIn > 0x7FFFFFFFull) { SRP_ERROR("drawBuffer", "Draw too large for the GPU path (%zu primitives)", nIn); return; }
	if (!ensureInit("drawBuffer")) return;
	runDraw(ib, vb, fb, sp, prim, start, count, nIn);
}

/* ------------------------------------------------------ multi-draw pass */

namespace {

struct PassLimits {
	unsigned long long in = 0, rows = 0, tiles = 0, pixels = 0;
};

/* Number of input primitives of a draw that a multi-draw pass can take, or 0
 * when the draw must go through drawBuffer (which also reports its errors):
 * filled triangles with an early-depth shader of the device set, buffers in
 * a valid range, framebuffer made by srpNewFramebuffer. */
size_t passInputs(const SRPGpuDraw& d)
{
	if (!d.vertexBuffer || !d.framebuffer || !d.program || !d.program->vs || !d.program->fs) return 0;
	if (!isTri(d.primitive) || d.count == 0) return 0;
	if (srpContext.raster.cullFace == SRP_FACE_FRONT_AND_BACK || srpContext.raster.polygonMode != SRP_POLYGON_MODE_FILL)
		return 0;
	const size_t size = d.indexBuffer ? d.indexBuffer->nIndices : d.vertexBuffer->nVertices;
	if (d.startIndex + d.count - 1 >= size || d.startIndex + d.count < d.startIndex) return 0;
	if (d.indexBuffer) {
		const SRPType t = d.indexBuffer->type;
		if (t != SRP_UINT8 && t != SRP_UINT16 && t != SRP_UINT32 && t != SRP_UINT64) return 0;
	}
	if (d.vertexBuffer->stride == 0 || d.vertexBuffer->stride > 1024) return 0;
	if (d.program->fs->mayOverwriteDepth) return 0;
	if (!lookupVS((void*) d.program->vs->shader) || !lookupFS((void*) d.program->fs->shader)) return 0;
	if (!fbFind(d.framebuffer)) return 0;
	const size_t n = d.primitive == SRP_PRIM_TRIANGLES ? d.count / 3 : (d.count >= 3 ? d.count - 2 : 0);
	return n <= 0x7FFFFFFFull ? n : 0;
}

/* Page-locked host staging that only grows. */
struct PinnedBuffer {
	void* ptr = nullptr;
	size_t bytes = 0;
	bool reserve(size_t need)
	{
		if (need <= bytes) return true;
		if (ptr) cudaFreeHost(ptr);
		ptr = nullptr;
		bytes = 0;
		const size_t nb = std::max(need, bytes + bytes / 2);
		if (cudaMallocHost(&ptr, nb) != cudaSuccess) { cudaGetLastError(); return false; }
		bytes = nb;
		return true;
	}
	template <class T> T* as() const { return (T*) ptr; }
};

/* The descriptors and prefix sums of a pass are staged in page-locked memory
 * so that their upload is asynchronous; a pass waits for its setup counters,
 * which follow the upload on the stream, before the staging is reused. */
PinnedBuffer passDesc;
std::vector<uint32_t> passPrefix;   /* in, v, t, blk: 4 x (n + 1) */


}  // namespace

/* One multi-draw pass over draws[idx[0..]] (all eligible, same shaders and
 * varying layout, distinct framebuffers). Returns false (after a message)
 * only on a CUDA failure; draws that hit a bad vertex index are re-run one
 * by one so that each reports as the ordinary draw does. */
/* After a pass (on the library's stream, with the first scratch set and the
 * shared front buffers): the next single draws' fronts wait for it. */
static void markPassDone()
{
	for (DrawSet& S : g.sets) cudaEventRecord(S.rasterDone, g.stream);
}

static bool runPass(const SRPGpuDraw* draws, const std::vector<size_t>& idx, const std::vector<size_t>& nInOf)
{
	const char* FN = "srpGpuDrawBatch";
	const size_t n = idx.size();
	const SRPShaderProgram* sp0 = draws[idx[0]].program;
	static DrawParams P;
	memset(&P, 0, sizeof P);
	if (g.tuneArmed) { cudaEventRecord(g.tuneStart, g.stream); g.tuneArmed = false; }
	/* a pass takes the next scratch set like a single draw; its front stages
	 * run on the front stream beside the previous pass's resolve and shading
	 * (except with learned shading, whose judge reshades on the library's
	 * stream: such a pass runs there whole) */
	DrawSet& S = g.sets[g.setNext];
	g.setNext ^= 1;
	/* after their downloads in flight; until the pass has been queued in
	 * full, downloads of its framebuffers go back to the library's stream */
	for (size_t k = 0; k < n; ++k)
		if (FbExtra* x = fbFind(draws[idx[k]].framebuffer)) {
			fbAfterDownloads(x);
			x->lastWrite = nullptr;
		}
	if (!buildLayout(sp0->vs, P.L)) return true;
	DrawState& st = P.st;
	st.frontFaceCW = srpContext.raster.frontFace == SRP_WINDING_CW;
	st.cullFace = srpContext.raster.cullFace;
	st.polygonMode = srpContext.raster.polygonMode;
	st.pointSize = srpContext.raster.pointSize;
	st.provokingFirst = srpContext.provokingVertexMode == SRP_PROVOKING_VERTEX_FIRST;
	st.scissorEnabled = srpContext.scissor.enabled;
	st.sx0 = srpContext.scissor.x; st.sx1 = srpContext.scissor.x + srpContext.scissor.width;
	st.sy0 = srpContext.scissor.y; st.sy1 = srpContext.scissor.y + srpContext.scissor.height;
	st.stencilEnabled = srpContext.stencil.enabled;
	const SRPStencilFaceState* fsrc[2] = { &srpContext.stencil.front, &srpContext.stencil.back };
	StencilFace* fdst[2] = { &st.front, &st.back };
	for (int i = 0; i < 2; ++i) {
		fdst[i]->func = fsrc[i]->func; fdst[i]->sfail = fsrc[i]->sfailOp; fdst[i]->dfail = fsrc[i]->dfailOp;
		fdst[i]->pass = fsrc[i]->passOp; fdst[i]->ref = fsrc[i]->ref; fdst[i]->mask = fsrc[i]->mask;
		fdst[i]->writeMask = fsrc[i]->writeMask;
	}
	st.depthTest = srpContext.depth.testEnable;
	st.depthWrite = srpContext.depth.writeEnable;
	st.depthOp = srpContext.depth.compareOp;
	st.earlyZ = 1;
	st.tile = kTile;
	P.vsId = lookupVS((void*) sp0->vs->shader);
	P.fsId = lookupFS((void*) sp0->fs->shader);
	P.heavyItems = g.tune.heavyItems;
	P.spinLimit = g.spinLimit;
	P.waitTest = g.waitTest;
	P.heavyCtasPerSM = g.tune.heavyCtasPerSM;
	P.prim = SRP_PRIM_TRIANGLES;

	/* descriptors and prefix sums */
	if (!passDesc.reserve(n * sizeof(DrawDesc))) {
		SRP_ERROR(FN, "cudaMallocHost failed for %zu draw descriptors", n);
		return false;
	}
	DrawDesc* desc = passDesc.as<DrawDesc>();
	passPrefix.assign(4 * (n + 1), 0u);
	uint32_t* pIn = passPrefix.data();
	uint32_t* pV = pIn + (n + 1);
	uint32_t* pT = pV + (n + 1);
	uint32_t* pB = pT + (n + 1);
	unsigned long long pix = 0;
	int maxStride = 4;
	std::vector<unsigned long long> pixBase(n);
	for (size_t k = 0; k < n; ++k) {
		const SRPGpuDraw& d = draws[idx[k]];
		SRPVertexBuffer* vb = (SRPVertexBuffer*) d.vertexBuffer;
		SRPIndexBuffer* ib = (SRPIndexBuffer*) d.indexBuffer;
		if (!uploadVB(vb) || (ib && !uploadIB(ib))) return false;
		FbExtra* fx = fbFind(d.framebuffer);
		DrawDesc& D = desc[k];
		memset(&D, 0, offsetof(DrawDesc, uniform));
		D.vertices = vb->dev.as<unsigned char>();
		D.indices = ib ? ib->dev.ptr : nullptr;
		D.indexSize = ib ? (int) ib->elemSize : 0;
		D.start = d.startIndex;
		D.count = d.count;
		D.nVertices = vb->nVertices;
		D.stride = (int) vb->stride;
		D.prim = d.primitive;
		D.W = (int) d.framebuffer->width;
		D.H = (int) d.framebuffer->height;
		D.tilesX = (D.W + kTile - 1) / kTile;
		D.tilesY = (D.H + kTile - 1) / kTile;
		D.color = fx->color; D.depth = fx->depth; D.stencil = fx->stencil;
		if (d.program->uniform) {
			SRPStdUniform u;
			memcpy(&u, d.program->uniform, sizeof u);
			if (u.texture) {
				SRPTexture* t = u.texture;
				if (!textureSync(t)) return false;
				u.texture = (SRPTexture*) t->desc;
			}
			memcpy(D.uniform, &u, sizeof u);
		} else {
			memset(D.uniform, 0, sizeof D.uniform);
		}
		maxStride = std::max(maxStride, D.stride);
		pIn[k + 1] = pIn[k] + (uint32_t) nInOf[k];
		pV[k + 1] = pV[k] + (uint32_t) D.nVertices;
		pT[k + 1] = pT[k] + (uint32_t) D.tilesX * (uint32_t) D.tilesY;
		pB[k + 1] = pB[k] + (uint32_t) ((D.nVertices + 127) / 128);
		pixBase[k] = pix;
		pix += d.framebuffer->size;
	}
	const uint32_t nIn = pIn[n], vRows = pV[n], numTiles = pT[n], vBlocks = pB[n];
	if (!S.passDesc.reserve(n * sizeof(DrawDesc), FN) || !S.passPrefix.reserve(passPrefix.size() * 4, FN) ||
	    !S.passPrimPrefix.reserve((n + 1) * 4, FN) || !S.passWinner.reserve(pix * 4 + 4, FN))
		return false;
	for (size_t k = 0; k < n; ++k) desc[k].winner = S.passWinner.as<int32_t>() + pixBase[k];
	P.draws = S.passDesc.as<DrawDesc>();
	P.nDraws = (uint32_t) n;
	P.inPrefix = S.passPrefix.as<uint32_t>();
	P.vPrefix = P.inPrefix + (n + 1);
	P.tPrefix = P.vPrefix + (n + 1);
	P.blkPrefix = P.tPrefix + (n + 1);
	P.primPrefix = S.passPrimPrefix.as<uint32_t>();
	P.nIn = (int) nIn;
	P.nVertices = vRows;
	P.minmax = S.minmax.as<unsigned long long>();
	P.ctr = S.ctr.as<DeviceCounters>();
	if (g.fbMode == SRP_GPU_FB_COHERENT)
		for (size_t k = 0; k < n; ++k) fbUpload(draws[idx[k]].framebuffer, fbFind(draws[idx[k]].framebuffer));

	const bool learned = learnedPrepare(P, kKindTri, false, (uint32_t) n, g.stream);
	const cudaStream_t fs = (g.overlap && !g.profiling && !learned) ? S.front : g.stream;
	/* the pass's resolve runs beside the previous pass's shading */
	const cudaStream_t rs = fs != g.stream ? g.resolveStream : g.stream;
	/* the front waits for the last draw that used this set (on the library's
	 * stream) and for the uploads of the draws' buffers since a front last
	 * waited for them: uploads complete in order on the copy stream, so the
	 * latest of them stands for all */
	if (fs != g.stream) cudaStreamWaitEvent(fs, S.rasterDone, 0);
	{
		cudaEvent_t latest = nullptr;
		unsigned long long latestSeq = 0;
		for (size_t k = 0; k < n; ++k) {
			const SRPGpuDraw& d = draws[idx[k]];
			SRPVertexBuffer* vb = (SRPVertexBuffer*) d.vertexBuffer;
			SRPIndexBuffer* ib = (SRPIndexBuffer*) d.indexBuffer;
			if (vb->pending && vb->ready && vb->seq > latestSeq) { latest = vb->ready; latestSeq = vb->seq; }
			if (ib && ib->pending && ib->ready && ib->seq > latestSeq) { latest = ib->ready; latestSeq = ib->seq; }
			vb->pending = false;
			if (ib) ib->pending = false;
		}
		if (latest) cudaStreamWaitEvent(fs, latest, 0);
	}
	/* descriptors and prefix sums go up on the front stream, ahead of the head */
	cudaMemcpyAsync(S.passDesc.ptr, desc, n * sizeof(DrawDesc), cudaMemcpyHostToDevice, fs);
	cudaMemcpyAsync(S.passPrefix.ptr, passPrefix.data(), passPrefix.size() * 4, cudaMemcpyHostToDevice, fs);
	uint32_t primCap = (uint32_t) std::min<unsigned long long>((unsigned long long) nIn + 4096, 0x3FFFFFFFu);
	uint32_t entryCap = (uint32_t) std::min<double>((double) nIn * g.entryRatio[kKindTri] + 4096, 4.0e9);
	const uint32_t keyBits = sortKeyBits(numTiles);
	bool drawn = false;
	for (int attempt = 0; attempt < 4 && !drawn; ++attempt) {
		const unsigned long long rows = (unsigned long long) vRows + g.clipRows;
		const size_t nw = (size_t) std::max(P.L.nWords, 1);
		const uint32_t blocks = (nIn + kSetupThreads - 1) / kSetupThreads;
		bool ok = S.clip.reserve(rows * 16, FN) && S.vary.reserve(rows * nw * 4, FN) &&
		          S.vset0.reserve((size_t) vRows * 16 + 16, FN) && S.vset1.reserve((size_t) vRows * 16 + 16, FN) &&
		          S.codes.reserve((size_t) vRows + 16, FN) &&
		          S.lookback.reserve((size_t) std::max(blocks, 1u) * 8, FN) &&
		          S.keys.reserve((size_t) entryCap * 4, FN) && S.vals.reserve((size_t) entryCap * 4, FN) &&
		          S.keys2.reserve((size_t) entryCap * 4, FN) && S.vals2.reserve((size_t) entryCap * 4, FN) &&
		          S.hist.reserve(sortHistWords(entryCap) * 4, FN) && S.partials.reserve(sortPartialWords(entryCap) * 4 + 64, FN) &&
		          S.big.reserve((size_t) g.bigCap * 16, FN) && S.table.reserve((size_t) g.tableCap * 4, FN) &&
		          S.clipSlot.reserve((size_t) nIn * 4 + 4, FN) &&
		          S.clipPolys.reserve((size_t) g.clipPolyCap * (1 + kMaxPoly) * 4, FN) &&
		          S.triR.reserve((size_t) primCap * sizeof(TriRaster), FN) &&
		          S.triA.reserve((size_t) primCap * sizeof(TriAttr), FN) && reserveClipFans(S, FN) &&
		          S.tileStart.reserve((size_t) (numTiles + 1) * 4, FN) && S.tileEnd.reserve((size_t) (numTiles + 1) * 4, FN) &&
		          S.heavy.reserve((size_t) (numTiles + 1) * 4, FN);
		if (!ok) return false;
		P.clip = S.clip.as<float4>();
		P.vset0 = S.vset0.as<float4>();
		P.vset1 = S.vset1.as<float4>();
		P.codes = S.codes.as<uint8_t>();
		P.vary = S.vary.as<uint32_t>();
		P.clipBase = vRows;
		P.clipCap = g.clipRows;
		P.triR = S.triR.as<TriRaster>();
		P.triA = S.triA.as<TriAttr>();
		P.primCap = primCap;
		P.keys = S.keys.as<uint32_t>();
		P.vals = S.vals.as<uint32_t>();
		P.entryCap = entryCap;
		P.bigJobs = S.big.as<uint4>();
		P.bigCap = g.bigCap;
		P.table = S.table.as<float>();
		P.tableCap = g.tableCap;
		P.clipSlot = S.clipSlot.as<uint32_t>();
		P.clipPolys = S.clipPolys.as<uint32_t>();
		P.clipPolyCap = g.clipPolyCap;
		setClipFans(P, S);
		P.lookback = S.lookback.as<unsigned long long>();
		P.tileStart = S.tileStart.as<uint32_t>();
		P.tileEnd = S.tileEnd.as<uint32_t>();

		auto head = [&]() {
			stageBegin();
			launchReset(P, fs);
			launchVertexMulti(P, vBlocks, maxStride, fs);
			stageEnd(SRP_GPU_STAGE_VERTEX, 2);
		};
		auto head2 = [&]() {
			stageBegin();
			cudaMemsetAsync(P.lookback, 0, (size_t) blocks * 8, fs);
			launchClipPrepassMulti(P, fs);
			launchSetupMulti(P, fs);
			launchCheck(P, fs);
			stageEnd(SRP_GPU_STAGE_SETUP, 3);
		};
		uint32_t* sk = nullptr;
		uint32_t* sv = nullptr;
		auto bin = [&]() {
			stageBegin();
			launchLambdaTablesMulti(P, g.bigJobsSeen[kKindTri], fs);
			launchBigEntriesMulti(P, g.bigJobsSeen[kKindTri], fs);
			sortEntries(P, keyBits, S.keys2.as<uint32_t>(), S.vals2.as<uint32_t>(), S.hist.as<uint32_t>(),
			            S.partials.as<uint32_t>(), &sk, &sv, fs);
			cudaMemsetAsync(P.tileStart, 0, (size_t) numTiles * 4, fs);
			cudaMemsetAsync(P.tileEnd, 0, (size_t) numTiles * 4, fs);
			launchTileRanges(P, sk, numTiles, fs);
			stageEnd(SRP_GPU_STAGE_BIN, 2 + 1 + (int) (keyBits / 8) + 1);
		};
		auto resolve = [&]() {
			stageBegin();
			launchResolveMulti(P, sv, numTiles, S.heavy.as<uint32_t>(), rs, g.auxStream, g.forkEvent, g.joinEvent);
			stageEnd(SRP_GPU_STAGE_RESOLVE, 3);
		};
		auto shade = [&]() {
			stageBegin();
			launchShadeMulti(P, numTiles, g.stream);
			stageEnd(SRP_GPU_STAGE_SHADE, 1);
		};
		runDrawSeq(graphKey(P, { vBlocks, (unsigned long long) maxStride, blocks, keyBits, numTiles,
		                         g.bigJobsSeen[kKindTri], (unsigned long long) (uintptr_t) g.stream,
		                         (unsigned long long) (uintptr_t) fs, (unsigned long long) (uintptr_t) rs }),
		           S, fs, rs, head, nullptr, head2, false, [] {}, bin, resolve, true, shade);
		if (fs == g.stream) markPassDone();
		g.launches += 5 + 2 + 1 + keyBits / 8 + 1 + 4;
		if (!cudaOk(cudaGetLastError(), FN, "launch")) return false;
		if (!cudaOk(cudaEventSynchronize(S.ctrEvent), FN, "kernel execution")) return false;
		const DeviceCounters c = *S.hostCtr;
		if (c.errors & kErrBadIndex) {
			/* some draw indexes past its vertex buffer: let each report alone */
			cudaStreamSynchronize(fs);
			cudaStreamSynchronize(g.stream);
			for (size_t k = 0; k < n; ++k) {
				const SRPGpuDraw& d = draws[idx[k]];
				drawBuffer(d.indexBuffer, d.vertexBuffer, d.framebuffer, d.program, d.primitive, d.startIndex, d.count);
			}
			return true;
		}
		if (c.errors & kErrSpin) { SRP_ERROR(FN, "Ordered-compaction wait timed out"); return false; }
		if (c.abort) {
			cudaStreamSynchronize(fs);
			cudaStreamSynchronize(g.stream);
			bool grew = false;
			if (c.clipVerts > g.clipRows) { g.clipRows = (uint32_t) std::min<unsigned long long>(c.clipVerts * 2, 0x7FFFFFFF); grew = true; }
			if (c.prims > primCap) { primCap = (uint32_t) std::min<unsigned long long>(c.prims + 1024, 0x3FFFFFFF); grew = true; }
			if (c.entries > entryCap) { entryCap = (uint32_t) std::min<double>(c.entries * 1.25 + 1024, 4.0e9); grew = true; }
			if (c.bigJobs > g.bigCap) { g.bigCap = (uint32_t) std::min<unsigned long long>(c.bigJobs * 2, 1u << 30); grew = true; }
			if (c.clipTris > g.clipPolyCap) { g.clipPolyCap = (uint32_t) std::min<unsigned long long>(c.clipTris * 2, 1u << 30); grew = true; }
			if (c.tableWords > g.tableCap) { g.tableCap = std::min<unsigned long long>(c.tableWords * 5 / 4 + 1024, 0xFFFFFFFFull); grew = true; }
			if (!grew) { SRP_ERROR(FN, "Scratch capacity exceeded"); return false; }
			++g.stats.drawRetries;
			continue;
		}
		g.entryRatio[kKindTri] = std::max(0.25, std::min(4096.0, (double) c.entries / (double) nIn * 1.25));
		g.bigJobsSeen[kKindTri] = (uint32_t) std::min<unsigned long long>(c.bigJobs, 1u << 30);
		g.stats.primitives += c.prims;
		g.stats.binEntries += c.entries;
		g.stats.clipOverflows += c.clipOverflow;
		g.profile.resolveTiles += numTiles;
		g.profile.resolveItems += c.entries;
		drawn = true;
	}
	if (!drawn) SRP_ERROR(FN, "Scratch capacity could not be sized for the pass");
	if (drawn && learned) {
		std::vector<uint8_t> redo(n);
		const uint8_t* redoDev = nullptr;
		if (learnedJudge((uint32_t) n, redo.data(), &redoDev, g.stream, P.ctr)) {
			P.fsId = P.judgeFs;
			P.redo = redoDev;
			stageBegin();
			launchShadeMulti(P, numTiles, g.stream);
			stageEnd(SRP_GPU_STAGE_SHADE, 1);
			++g.launches;
			P.redo = nullptr;
		}
	}
	g.stats.draws += n;
	if (drawn) {
		unsigned long long seq = 0;
		const cudaEvent_t e = drawWriteEvent(seq);
		for (size_t k = 0; k < n; ++k)
			if (FbExtra* x = fbFind(draws[idx[k]].framebuffer)) {
				x->lastWrite = e;
				x->lastWriteSeq = seq;
			}
	}
	if (g.fbMode == SRP_GPU_FB_COHERENT)
		for (size_t k = 0; k < n; ++k) fbDownload(draws[idx[k]].framebuffer, fbFind(draws[idx[k]].framebuffer));
	if (fs == g.stream) markPassDone();
	return true;
}

extern "C" {

void srpDrawVertexBuffer(const SRPVertexBuffer* vb, const SRPFramebuffer* fb, const SRPShaderProgram* sp,
                         SRPPrimitive prim, size_t start, size_t count)
{
	drawBuffer(nullptr, vb, fb, sp, prim, start, count);
}

void srpDrawIndexBuffer(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                        const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count)
{
	drawBuffer(ib, vb, fb, sp, prim, start, count);
}

constexpr size_t kPassDraws = 1024;

void srpGpuDrawBatch(const SRPGpuDraw* draws, size_t n)
{
	if (!draws || n == 0) return;
	if (!ensureInit("srpGpuDrawBatch")) return;
	/* limits of one pass: 32-bit input, row and tile numbers, 24-bit tile keys */
	const unsigned long long kMaxIn = 0x7FFFFFFFull, kMaxRows = 0x7FFFFFFFull - (1ull << 24), kMaxTiles = 1ull << 24;
	size_t i = 0;
	std::vector<size_t> idx, nInOf;
	std::unordered_set<const SRPFramebuffer*> fbs;
	while (i < n) {
		idx.clear(); nInOf.clear(); fbs.clear();
		unsigned long long in = 0, rows = 0, tiles = 0;
		VaryingLayout L0;
		int vs0 = 0, fs0 = 0;
		const SRPVertexShader* vsSeen = nullptr;   /* a vertex shader whose layout equals L0 */
		size_t j = i;
		for (; j < n; ++j) {
			const SRPGpuDraw& d = draws[j];
			const size_t k = passInputs(d);
			if (!k) break;
			const int vs = lookupVS((void*) d.program->vs->shader), fs = lookupFS((void*) d.program->fs->shader);
			if (d.program->vs != vsSeen || idx.empty()) {
				VaryingLayout L;
				if (!buildLayout(d.program->vs, L)) break;
				if (idx.empty()) L0 = L;
				else if (memcmp(&L, &L0, sizeof L) != 0) break;
				vsSeen = d.program->vs;
			}
			if (idx.empty()) { vs0 = vs; fs0 = fs; }
			else if (vs != vs0 || fs != fs0) break;
			if (!fbs.insert(d.framebuffer).second) break;
			const unsigned long long t = (unsigned long long) ((d.framebuffer->width + kTile - 1) / kTile) *
			                             ((d.framebuffer->height + kTile - 1) / kTile);
			if (in + k > kMaxIn || rows + d.vertexBuffer->nVertices > kMaxRows || tiles + t >= kMaxTiles) break;
			/* passes of at most kPassDraws draws, so that the front stages of
			 * one pass overlap the resolve and shading of the previous one */
			if (idx.size() >= kPassDraws) break;
			in += k; rows += d.vertexBuffer->nVertices; tiles += t;
			idx.push_back(j); nInOf.push_back(k);
		}
		if (idx.size() >= 2) {
			for (size_t k : idx) warnExcess(draws[k].primitive, draws[k].count);
			if (!runPass(draws, idx, nInOf)) return;
			i = j;
		} else {
			const SRPGpuDraw& d = draws[i];
			drawBuffer(d.indexBuffer, d.vertexBuffer, d.framebuffer, d.program, d.primitive, d.startIndex, d.count);
			++i;
		}
	}
}

/* ------------------------------------------------------- stream and stats */

void srpGpuSetStream(void* stream)
{
	if (!ensureInit("srpGpuSetStream")) return;
	cudaStreamSynchronize(g.downloadStream);
	cudaStreamSynchronize(g.copyStream);
	syncFronts();
	cudaStreamSynchronize(g.resolveStream);
	cudaStreamSynchronize(g.stream);
	g.stream = stream ? (cudaStream_t) stream : g.ownStream;
	g.rsDirty = true;
}

void* srpGpuGetStream(void) { return ensureInit("srpGpuGetStream") ? (void*) g.stream : nullptr; }

int srpGpuSynchronize(void)
{
	if (!g.init) return 0;
	cudaStreamSynchronize(g.downloadStream);
	cudaStreamSynchronize(g.copyStream);
	syncFronts();
	cudaStreamSynchronize(g.resolveStream);
	return cudaOk(cudaStreamSynchronize(g.stream), "srpGpuSynchronize", "kernel execution") ? 0 : 1;
}

void srpGpuGetStats(SRPGpuStats* s)
{
	if (!g.init) { memset(s, 0, sizeof *s); return; }
	const unsigned long long frags = readCounters();
	*s = g.stats;
	s->fragments = frags;
	s->kernelLaunches = g.launches;
}

void srpGpuResetStats(void)
{
	if (!g.init) return;
	syncFronts();
	cudaStreamSynchronize(g.resolveStream);
	cudaStreamSynchronize(g.stream);
	for (DrawSet& S : g.sets) cudaMemset(S.ctr.ptr, 0, sizeof(DeviceCounters));
	g.stats = SRPGpuStats();
	g.launches = 0;
}

void srpGpuSetProfiling(int enable) { g.profiling = enable != 0; }

void srpGpuSetDrawGraphs(int enable) { g.graphs = enable != 0; }

void srpGpuSetDrawOverlap(int enable)
{
	if (!ensureInit("srpGpuSetDrawOverlap")) return;
	syncFronts();
	cudaStreamSynchronize(g.resolveStream);
	g.overlap = enable != 0;
}

void srpGpuGetTuning(SRPGpuTuning* t) { *t = g.tune; }

void srpGpuSetTuning(const SRPGpuTuning* t)
{
	g.tune.heavyItems = t->heavyItems;
	g.tune.heavyCtasPerSM = t->heavyCtasPerSM >= 1 && t->heavyCtasPerSM <= 3 ? t->heavyCtasPerSM : 3;
}

/* Online autotuning of a frame loop: kTuneFrames frames per candidate, the
 * first of which captures the graphs of the new tuning; the others are timed
 * one by one and the candidate scores its fastest frame. */
namespace {
constexpr int kTuneFrames = 4;
struct FrameTuner {
	int state = -1;          /* -1 idle, 0 .. kTuneFrames * candidates - 1 running, -2 done */
	cudaEvent_t stop = nullptr;   /* the start event is g.tuneStart */
	float best = -1.0f;
	SRPGpuTuning bestTune = { 96, 3 };
} tuner;
const uint32_t kTuneThresholds[] = { 32, 64, 96, 192, 384 };
constexpr int kTuneCandidates = 5 * 3;
SRPGpuTuning tuneCandidate(int i) { return SRPGpuTuning{ kTuneThresholds[i / 3], (uint32_t) (i % 3 + 1) }; }
}  // namespace

int srpGpuAutotuneFrame(void)
{
	if (tuner.state == -2 || !ensureInit("srpGpuAutotuneFrame")) return 0;
	if (!tuner.stop) { g.tuneStart = takeEvent(); tuner.stop = takeEvent(); }
	if (tuner.state >= 0 && tuner.state % kTuneFrames != 0) {
		/* a timed frame just ended */
		cudaEventRecord(tuner.stop, g.stream);
		float ms = 0.0f;
		if (cudaEventSynchronize(tuner.stop) == cudaSuccess && cudaEventElapsedTime(&ms, g.tuneStart, tuner.stop) == cudaSuccess &&
		    (tuner.best < 0.0f || ms < tuner.best)) {
			tuner.best = ms;
			tuner.bestTune = g.tune;
		}
	}
	++tuner.state;
	if (tuner.state >= kTuneFrames * kTuneCandidates) {
		g.tune = tuner.bestTune;
		tuner.state = -2;
		return 0;
	}
	g.tune = tuneCandidate(tuner.state / kTuneFrames);
	/* the timed frame starts with its first draw (not now: the caller may
	 * clear or upload first) */
	g.tuneArmed = tuner.state % kTuneFrames != 0;
	return 1;
}

void srpGpuAutotuneReset(void)
{
	tuner.state = -1;
	tuner.best = -1.0f;
	g.tuneArmed = false;
}

int srpGpuAutotune(const SRPGpuDraw* draws, size_t n, int repeats, SRPGpuTuning* best)
{
	if (!draws || !n || !ensureInit("srpGpuAutotune")) return -1;
	static const uint32_t thresholds[] = { 32, 64, 96, 192, 384 };
	cudaEvent_t e0 = takeEvent(), e1 = takeEvent();
	const SRPGpuTuning start = g.tune;
	SRPGpuTuning top = start;
	float topMs = -1.0f;
	srpGpuDrawBatch(draws, n);   /* warm-up: sizes the scratch */
	for (uint32_t th : thresholds)
		for (uint32_t per = 1; per <= 3; ++per) {
			g.tune.heavyItems = th;
			g.tune.heavyCtasPerSM = per;
			srpGpuDrawBatch(draws, n);   /* first run captures the graphs for this tuning */
			float ms = 0.0f;
			cudaEventRecord(e0, g.stream);
			for (int r = 0; r < (repeats > 0 ? repeats : 1); ++r) srpGpuDrawBatch(draws, n);
			cudaEventRecord(e1, g.stream);
			if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
				g.tune = start;
				SRP_ERROR("srpGpuAutotune", "timing failed");
				return -1;
			}
			if (topMs < 0.0f || ms < topMs) { topMs = ms; top = g.tune; }
		}
	g.eventPool.push_back(e0);
	g.eventPool.push_back(e1);
	g.tune = top;
	if (best) *best = top;
	return 0;
}

void srpGpuGetProfile(SRPGpuProfile* out)
{
	if (g.init) {
		cudaStreamSynchronize(g.stream);
		for (auto& p : g.pending) {
			float ms = 0.f;
			if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) g.profile.ms[p.first] += ms;
			g.eventPool.push_back(p.second.first);
			g.eventPool.push_back(p.second.second);
		}
		g.pending.clear();
	}
	*out = g.profile;
}

void srpGpuResetProfile(void)
{
	SRPGpuProfile tmp;
	srpGpuGetProfile(&tmp);
	g.profile = SRPGpuProfile();
}

void srpGpuSetTileSize(int tileSize)
{
	if (tileSize != kTile) SRP_ERROR("srpGpuSetTileSize", "Only %d-pixel tiles are built into this library", kTile);
}

void srpGpuSetWaitLimit(uint32_t iterations) { g.spinLimit = iterations; }

void srpGpuSetTileCopies(unsigned parts)
{
	g.tma = parts & (SRP_GPU_TILE_COPY_RESOLVE_LOAD | SRP_GPU_TILE_COPY_RESOLVE_STORE | SRP_GPU_TILE_COPY_SHADE);
}

void srpGpuSetWaitTest(uint32_t flags) { g.waitTest = flags & (kWaitTestSetup | kWaitTestLearned); }

void srpGpuSetEntryEstimate(double entriesPerPrimitive)
{
	const double r = entriesPerPrimitive < 0.0 ? 0.0 : std::min(entriesPerPrimitive, 4096.0);
	for (double& e : g.entryRatio) e = r;
}

}  // extern "C"

/* ------------------------------------------- for the fixed-scratch draw */

namespace srpg {

int fixedDrawPrepare(DrawParams& P, const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                     const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count, FixedDrawInfo& info)
{
	const char* FN = "srpGpuDrawFixedScratch";
	/* validation and early returns of drawBuffer (src/pipeline/draw.c:63-82) */
	if (count == 0) return 1;
	const size_t end = start + count - 1;
	const size_t size = ib ? ib->nIndices : vb->nVertices;
	if (end >= size) {
		SRP_ERROR("checkOOB", ib ? "Attempt to OOB access index buffer (read) at indices %zu-%zu (size: %zu)\n"
		                         : "Attempt to OOB access vertex buffer (read) at indices %zu-%zu (size: %zu)\n",
		          start, end, size);
		return -1;
	}
	size_t nIn = 0;
	if (isTri(prim)) {
		if (srpContext.raster.cullFace == SRP_FACE_FRONT_AND_BACK) return 1;
		warnExcess(prim, count);
		nIn = prim == SRP_PRIM_TRIANGLES ? count / 3 : (count >= 3 ? count - 2 : 0);
		if (srpContext.raster.polygonMode != SRP_POLYGON_MODE_FILL && srpContext.raster.polygonMode != SRP_POLYGON_MODE_LINE &&
		    srpContext.raster.polygonMode != SRP_POLYGON_MODE_POINT) {
			SRP_ERROR("assembleTrianglesGeneric", "Unexpected srpContext.raster.polygonMode (%i)", (int) srpContext.raster.polygonMode);
			return -1;
		}
	} else if (isLine(prim)) {
		warnExcess(prim, count);
		nIn = prim == SRP_PRIM_LINES ? count / 2 : (count != 1 ? (prim == SRP_PRIM_LINE_STRIP ? count - 1 : count) : 0);
	} else if (prim == SRP_PRIM_POINTS) {
		if (srpContext.raster.pointSize <= 0.) return 1;
		nIn = count;
	} else {
		SRP_ERROR("drawBuffer", "Unknown primitive type: %i", (int) prim);
		return -1;
	}
	if (nIn == 0) return 1;
	if (nIn > 0x7FFFFFFFull) { SRP_ERROR(FN, "Draw too large for the GPU path (%zu primitives)", nIn); return -1; }
	/* what the ordinary draw would set up by allocating */
	if (!g.init) { SRP_ERROR(FN, "The library is not initialised: create the framebuffer with srpNewFramebuffer first"); return -1; }
	/* the draw reads its counters back to the host partway through, which no
	 * stream capture allows: reject it before anything is queued or changed */
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	const cudaError_t ce = cudaStreamIsCapturing(g.stream, &cap);
	if (ce != cudaSuccess) cudaGetLastError();
	if (ce != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
		SRP_ERROR(FN, "Called while the library's stream is being captured: a fixed-scratch draw waits for its "
		              "counters mid-draw, so no call can be part of a CUDA graph capture");
		return -1;
	}
	FbExtra* fx = fbFind(fb);
	if (!fx) { SRP_ERROR(FN, "Framebuffer was not created by srpNewFramebuffer"); return -1; }
	if (vb->dirty || (!vb->dev.ptr && vb->nBytes)) {
		SRP_ERROR(FN, "Vertex buffer is not in device memory (its data was copied while no GPU was usable)");
		return -1;
	}
	if (ib && (ib->dirty || (!ib->dev.ptr && ib->nBytes))) {
		SRP_ERROR(FN, "Index buffer is not in device memory (its data was copied while no GPU was usable)");
		return -1;
	}
	const int vsId = lookupVS((void*) sp->vs->shader);
	const int fsId = lookupFS((void*) sp->fs->shader);
	if (!vsId || !fsId) {
		SRP_ERROR(FN, "Shader has no GPU implementation; map it with srpGpuRegisterVertexShader/FragmentShader");
		return -1;
	}
	if (vb->stride == 0 || vb->stride > 1024) {
		SRP_ERROR(FN, "GPU path supports vertex strides of 1..1024 bytes (got %zu)", vb->stride);
		return -1;
	}
	memset(&P, 0, sizeof P);
	if (!buildLayout(sp->vs, P.L)) return -1;
	/* state snapshot, as in runDraw */
	DrawState& st = P.st;
	st.W = (int) fb->width; st.H = (int) fb->height;
	st.frontFaceCW = srpContext.raster.frontFace == SRP_WINDING_CW;
	st.cullFace = srpContext.raster.cullFace;
	st.polygonMode = srpContext.raster.polygonMode;
	st.pointSize = srpContext.raster.pointSize;
	st.provokingFirst = srpContext.provokingVertexMode == SRP_PROVOKING_VERTEX_FIRST;
	st.scissorEnabled = srpContext.scissor.enabled;
	st.sx0 = srpContext.scissor.x; st.sx1 = srpContext.scissor.x + srpContext.scissor.width;
	st.sy0 = srpContext.scissor.y; st.sy1 = srpContext.scissor.y + srpContext.scissor.height;
	st.stencilEnabled = srpContext.stencil.enabled;
	const SRPStencilFaceState* fsrc[2] = { &srpContext.stencil.front, &srpContext.stencil.back };
	StencilFace* fdst[2] = { &st.front, &st.back };
	for (int i = 0; i < 2; ++i) {
		fdst[i]->func = fsrc[i]->func; fdst[i]->sfail = fsrc[i]->sfailOp; fdst[i]->dfail = fsrc[i]->dfailOp;
		fdst[i]->pass = fsrc[i]->passOp; fdst[i]->ref = fsrc[i]->ref; fdst[i]->mask = fsrc[i]->mask;
		fdst[i]->writeMask = fsrc[i]->writeMask;
	}
	st.depthTest = srpContext.depth.testEnable;
	st.depthWrite = srpContext.depth.writeEnable;
	st.depthOp = srpContext.depth.compareOp;
	st.earlyZ = !sp->fs->mayOverwriteDepth;
	st.tile = kTile;
	st.tilesX = (st.W + kTile - 1) / kTile;
	st.tilesY = (st.H + kTile - 1) / kTile;
	if (sp->uniform) {
		SRPStdUniform u;
		memcpy(&u, sp->uniform, sizeof u);
		if (u.texture) {
			SRPTexture* t = u.texture;
			/* textures get their device texels when they are created */
			if (!t->texels || !t->desc) { SRP_ERROR(FN, "Texture has no device texels"); return -1; }
			if (!textureSync(t)) return -1;
			u.texture = (SRPTexture*) t->desc;
		}
		memcpy(P.uniform, &u, sizeof u);
	}
	P.vsId = vsId;
	P.fsId = fsId;
	P.heavyItems = g.tune.heavyItems;
	P.spinLimit = g.spinLimit;
	P.waitTest = g.waitTest;
	P.heavyCtasPerSM = g.tune.heavyCtasPerSM;
	P.prim = prim;
	P.start = start;
	P.count = count;
	P.nIn = (int) nIn;
	P.vertices = vb->dev.as<unsigned char>();
	P.nVertices = vb->nVertices;
	P.stride = (int) vb->stride;
	if (ib) {
		if (ib->type != SRP_UINT8 && ib->type != SRP_UINT16 && ib->type != SRP_UINT32 && ib->type != SRP_UINT64) {
			SRP_ERROR("indexIndexBuffer", "Unexpected type (%i)", (int) ib->type);
			return -1;
		}
		P.indices = ib->dev.ptr;
		P.indexSize = (int) ib->elemSize;
	}
	P.color = fx->color;
	P.depth = fx->depth;
	P.stencil = fx->stencil;
	const int mode = isTri(prim) ? st.polygonMode : (isLine(prim) ? SRP_POLYGON_MODE_LINE : SRP_POLYGON_MODE_POINT);
	info.stream = g.stream;
	fbOtherWrite(fx);
	g.rsDirty = true;  /* its resolve writes the planes on the library's stream */
	/* the uploads of its buffers, on the copy stream */
	if (vb->ready) cudaStreamWaitEvent(g.stream, vb->ready, 0);
	if (ib && ib->ready) cudaStreamWaitEvent(g.stream, ib->ready, 0);
	info.nIn = nIn;
	info.outPer = isTri(prim) && mode != SRP_POLYGON_MODE_FILL ? 3 : 1;
	info.numTiles = (uint32_t) st.tilesX * (uint32_t) st.tilesY;
	info.pixels = fb->size;
	info.kind = mode == SRP_POLYGON_MODE_FILL ? kKindTri : mode == SRP_POLYGON_MODE_LINE ? kKindLineFrag : kKindPoint;
	info.triangles = isTri(prim);
	info.late = sp->fs->mayOverwriteDepth && shadeSupportsLateDepth(fsId);
	info.coherent = g.fbMode == SRP_GPU_FB_COHERENT;
	return 0;
}

void fixedDrawError(const char* fn, const char* fmt, ...)
{
	if (!srpContext.messageCallback.func) return;
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	srpContext.messageCallback.func(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, fn, buf,
	                                srpContext.messageCallback.userParameter);
}

void fixedDrawUpload(const SRPFramebuffer* fb)
{
	if (FbExtra* x = fbFind(fb)) fbUpload(fb, x);
}

void fixedDrawDownload(const SRPFramebuffer* fb)
{
	if (FbExtra* x = fbFind(fb)) fbDownload(fb, x);
}

void learnedError(const char* fmt, ...)
{
	if (!srpContext.messageCallback.func) return;
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	srpContext.messageCallback.func(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpGpuLearnedShading", buf,
	                                srpContext.messageCallback.userParameter);
}

int learnedShaderId(void* fragmentShader) { return lookupFS(fragmentShader); }

void fixedDrawAccount(const DeviceCounters& c, unsigned launches)
{
	g.stats.primitives += c.prims;
	g.stats.binEntries += c.entries;
	g.stats.clipOverflows += c.clipOverflow;
	++g.stats.draws;
	g.launches += launches;
}

}  // namespace srpg
