/* srp-gb300: additions to the srp API for the GPU implementation.
 *
 * Nothing here has a counterpart in kitrofimov/srp; the reference API itself
 * (srp/srp.h) is implemented unchanged. These entry points cover what a GPU
 * build needs beyond it: mapping host shader functions to device shaders,
 * controlling when the framebuffer's host mirrors are refreshed, choosing the
 * CUDA stream, and reading counters. All are plain C (extern "C"). */
#pragma once

#include <stddef.h>
#include <stdint.h>
#include "srp/srp.h"
#include "srp/shaderlib.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ shaders */

/** Map a host vertex shader function to a built-in device shader. The
 *  built-in host functions of srp/shaderlib.h are mapped already. */
void srpGpuRegisterVertexShader(void (*hostShader)(SRPVertexShaderIn*, SRPVertexShaderOut*),
                                SRPGpuVertexShaderId deviceShader);
/** Map a host fragment shader function to a built-in device shader. */
void srpGpuRegisterFragmentShader(void (*hostShader)(SRPFragmentShaderIn*, SRPFragmentShaderOut*),
                                  SRPGpuFragmentShaderId deviceShader);

/* -------------------------------------------------------- framebuffer */

typedef enum SRPGpuFramebufferMode
{
	/** Default, for unmodified srp programs: every draw first uploads the
	 *  host planes (which the program may have edited) and afterwards
	 *  downloads the result, and every clear is mirrored, so the public
	 *  color/depth/stencil arrays are always current. */
	SRP_GPU_FB_COHERENT = 0,
	/** The device planes are authoritative. Host arrays are refreshed only by
	 *  srpGpuFramebufferSync and pushed only by srpGpuFramebufferUpload. */
	SRP_GPU_FB_DEVICE = 1
} SRPGpuFramebufferMode;

void srpGpuSetFramebufferMode(SRPGpuFramebufferMode mode);
SRPGpuFramebufferMode srpGpuGetFramebufferMode(void);

/** Copy the device planes into the host arrays (waits for the GPU). */
void srpGpuFramebufferSync(const SRPFramebuffer* fb);
/** Copy the host arrays to the device planes. */
void srpGpuFramebufferUpload(const SRPFramebuffer* fb);
/** Sync the framebuffer and write its colour plane as a PNG (RGBA8, alpha
 *  255, top row first): what the reference's test harness does with
 *  stb_image_write (tests/utils/save.c:3-34), without the dependency.
 *  Returns 0 on success. */
int srpGpuSaveFramebufferPNG(const SRPFramebuffer* fb, const char* path);

#define SRP_GPU_FILL_COLOR   1u
#define SRP_GPU_FILL_DEPTH   2u
#define SRP_GPU_FILL_STENCIL 4u
/** Fill the selected device planes with constants (stream-ordered). */
void srpGpuFramebufferFill(const SRPFramebuffer* fb, uint32_t color, float depth, uint8_t stencil,
                           unsigned planes);
/** srpGpuFramebufferFill of n framebuffers in one launch. */
void srpGpuFramebufferFillBatch(const SRPFramebuffer* const* fbs, size_t n, uint32_t color, float depth,
                                uint8_t stencil, unsigned planes);

/* ------------------------------------------- asynchronous transfers */

/* Stream-ordered versions of the transfers for programs that move many
 * buffers per frame: they only enqueue the copy and return. The host memory
 * they read or write belongs to the library until the next srpGpuSynchronize
 * (the caller must not change a source, nor read a destination, before it);
 * from page-locked memory the copies then run at the host link's speed
 * without a round trip per call. None has a counterpart in the reference. */

/** srpVertexBufferCopyData without waiting for the copy. Copies run in
 *  order on a copy stream of the library; a draw that reads the buffer waits
 *  for its copy, and nothing else does. A copy into a buffer that earlier
 *  draws read does not wait for them either: every draw call returns only
 *  after its device stages have read its vertex and index buffers. */
void srpGpuVertexBufferCopyDataAsync(SRPVertexBuffer* buffer, size_t stride, size_t nBytes, const void* data);
/** srpIndexBufferCopyData without waiting for the copy. */
void srpGpuIndexBufferCopyDataAsync(SRPIndexBuffer* buffer, SRPType type, size_t nBytes, const void* data);
/** srpGpuFramebufferSync without waiting: the host arrays are current after
 *  the next srpGpuSynchronize. */
void srpGpuFramebufferSyncAsync(const SRPFramebuffer* fb);

/** Many srpGpuVertexBufferCopyDataAsync calls in one: buffer i takes
 *  nBytes[i] bytes of stride strides[i] from data[i]. Sources the device can
 *  reach (page-locked memory, or any host memory where the device has
 *  pageable-memory access) are copied by one gather kernel per 256 buffers
 *  on the copy stream, at the host link's speed and without a driver call
 *  per buffer; other sources take the single-buffer path. */
void srpGpuVertexBufferCopyDataBatchAsync(SRPVertexBuffer* const* buffers, const size_t* strides, const size_t* nBytes,
                                          const void* const* data, size_t n);
/** Many srpGpuIndexBufferCopyDataAsync calls in one, as above. */
void srpGpuIndexBufferCopyDataBatchAsync(SRPIndexBuffer* const* buffers, const SRPType* types, const size_t* nBytes,
                                         const void* const* data, size_t n);
/** Many srpGpuFramebufferSyncAsync calls in one: framebuffers last written by
 *  the same draw or batch pass come back by one gather kernel, after that
 *  draw or pass only, beside later ones. The host arrays are current after
 *  the next srpGpuSynchronize. */
void srpGpuFramebufferSyncBatchAsync(const SRPFramebuffer* const* fbs, size_t n);

/* ----------------------------------------------------- batched draws */

/** One draw of srpGpuDrawBatch: the arguments of srpDrawIndexBuffer
 *  (indexBuffer not NULL) or srpDrawVertexBuffer (indexBuffer NULL). */
typedef struct SRPGpuDraw
{
	const SRPIndexBuffer* indexBuffer;
	const SRPVertexBuffer* vertexBuffer;
	const SRPFramebuffer* framebuffer;
	const SRPShaderProgram* program;
	SRPPrimitive primitive;
	size_t startIndex;
	size_t count;
} SRPGpuDraw;

/** Issue n draws in one call. It has no counterpart in kitrofimov/srp; the
 *  result is exactly that of calling srpDrawIndexBuffer / srpDrawVertexBuffer
 *  for draws[0], draws[1], ... in order, with the context state of the call.
 *
 *  Runs of consecutive draws that are filled triangles with an early-depth
 *  device shader, share the vertex shader, fragment shader and varying
 *  layout, and target different framebuffers are rendered as one multi-draw
 *  pass: one set of kernel launches for all of them, whatever their sizes.
 *  Every other draw, including any draw the ordinary path would reject with
 *  a message, is issued through the ordinary path at its place in the order. */
void srpGpuDrawBatch(const SRPGpuDraw* draws, size_t n);

/** Tuning of the resolve stage. Tiles with more than heavyItems (tile, item)
 *  pairs are resolved by a 256-thread CTA each (8 warps per tile), the others
 *  by one warp; the CTA kernel runs heavyCtasPerSM (1..3) CTAs per SM. The
 *  tile itself is fixed at 8 x 8 pixels: the exact resolve's 64-bit coverage
 *  masks depend on it. */
typedef struct SRPGpuTuning
{
	uint32_t heavyItems;
	uint32_t heavyCtasPerSM;
} SRPGpuTuning;

void srpGpuGetTuning(SRPGpuTuning* tuning);
void srpGpuSetTuning(const SRPGpuTuning* tuning);

/** Autotuner: draws the batch (srpGpuDrawBatch) `repeats` times under each
 *  candidate tuning (heavyItems 32, 64, 96, 192, 384 x heavyCtasPerSM 1..3),
 *  times it with CUDA events, and keeps the fastest as the library's tuning
 *  (also returned in best). The framebuffers are drawn into repeatedly:
 *  prepare them again afterwards. Returns 0 on success. */
int srpGpuAutotune(const SRPGpuDraw* draws, size_t n, int repeats, SRPGpuTuning* best);

/** Online autotuner for a frame loop: call once after each frame's draws.
 *  Over the next 60 frames it tries the same candidates as srpGpuAutotune,
 *  four frames each (the last three timed one by one with CUDA events, from
 *  the frame's first draw to this call), then keeps the candidate with the
 *  fastest frame. Returns 1 while tuning, 0 once a tuning has been chosen
 *  (and on every later call, until srpGpuAutotuneReset). */
int srpGpuAutotuneFrame(void);
void srpGpuAutotuneReset(void);

/* --------------------------------------------------- learned shading */

/* A small MLP that stands in for an expensive fragment shader. None of this
 * has a counterpart in kitrofimov/srp. The network maps a 6-band sin/cos
 * encoding of the fragment's world position, unit normal and unit view
 * direction (108 inputs) through three hidden layers of 64 ReLU units to
 * RGB. It learns from fragments the shader itself shaded, is trained on the
 * GPU (fp32, Adam), and shades on the tensor cores (bf16 weights, fp32
 * accumulation). Coverage, depth, stencil and the visible fragment never
 * depend on it: only the colour of the visible fragment does. The one
 * shader with a learned stand-in is srpFsMarble (world-space varyings of
 * srpVsWorld). */
typedef struct SRPGpuMlp SRPGpuMlp;

/** A network with seeded random weights and room for sampleCapacity
 *  captured fragments. */
SRPGpuMlp* srpGpuMlpCreate(uint64_t seed, size_t sampleCapacity);
void srpGpuMlpFree(SRPGpuMlp* mlp);

/** While set, every draw shaded by `target` records 1 of every `every`
 *  shaded pixels (position, normal, view direction, colour) into mlp, up to
 *  its capacity. mlp NULL stops the capture. */
void srpGpuMlpCapture(SRPGpuMlp* mlp, void (*target)(SRPFragmentShaderIn*, SRPFragmentShaderOut*), uint32_t every);
size_t srpGpuMlpSampleCount(const SRPGpuMlp* mlp);
/** Append samples given by the host: 12 floats each (position, normal, view
 *  direction, RGB). Returns 0, or -1 beyond the capacity. */
int srpGpuMlpAddSamples(SRPGpuMlp* mlp, const float* samples, size_t n);

/** Train on the samples: `steps` Adam steps (cosine-decayed rate from
 *  learningRate) over random batches of `batch`. Returns the mean squared
 *  error of the last batch, or a negative value on failure. */
float srpGpuMlpTrain(SRPGpuMlp* mlp, int steps, int batch, float learningRate);

/** Draws whose fragment shader is `target` are shaded by mlp. 1 pixel in
 *  judgeEvery is also shaded by `target`; a draw whose PSNR over those
 *  pixels (between the two images' stored 8-bit colour channels, scaled to
 *  [0, 1]) is below minPsnrDb is shaded again by `target` alone. mlp NULL
 *  turns learned shading off. */
void srpGpuSetLearnedShading(void (*target)(SRPFragmentShaderIn*, SRPFragmentShaderOut*), SRPGpuMlp* mlp,
                             float minPsnrDb, uint32_t judgeEvery);

typedef struct SRPGpuLearnedStats
{
	uint64_t draws;              /* learned-shaded draws */
	uint64_t fallbacks;          /* of them, shaded again by the target shader */
	uint64_t judgedDraws;        /* draws with at least one judged pixel */
	uint64_t judgedChannels;     /* colour channels compared with the target */
	double squaredError;         /* summed over the judged channels (range [0, 1]) */
	double lastPsnrDb, minPsnrDb;
	float maxChannelError;
	/* judged draws by PSNR: < 20, 20-25, 25-30, 30-35, 35-40, >= 40 dB */
	uint64_t psnrHistogram[6];
} SRPGpuLearnedStats;

/** Statistics since the last reset (reading them does not wait for the GPU:
 *  every learned-shaded draw is judged before it returns). */
void srpGpuGetLearnedStats(SRPGpuLearnedStats* stats);
void srpGpuResetLearnedStats(void);

/** The network's parameters as one fp32 vector (W1 [108][64], b1, W2 [64][64],
 *  b2, W3 [64][64], b3, W4 [64][3], b4), for inspection and tests. */
size_t srpGpuMlpParamCount(void);
void srpGpuMlpGetParams(const SRPGpuMlp* mlp, float* params);
void srpGpuMlpSetParams(SRPGpuMlp* mlp, const float* params);
/** RGB (unclamped) of n samples: fp32 on CUDA cores (tensorCores 0) or, as
 *  in the shading path, bf16 tcgen05 MMA with the accumulators in tensor
 *  memory (1). Returns 0 on success. */
int srpGpuMlpEvaluate(SRPGpuMlp* mlp, const float* samples, size_t n, float* rgb, int tensorCores);
/** Gradient of the mean squared error over n samples (in order) with
 *  respect to the parameters, and the summed squared error. */
int srpGpuMlpGradients(SRPGpuMlp* mlp, const float* samples, size_t n, float* grad, double* sse);

/* ------------------------------------------------- fixed-scratch draw */

/** Size of the device array that srpGpuDrawFixedScratch takes its scratch
 *  from (64 MiB). */
#define SRP_GPU_FIXED_SCRATCH_BYTES (64u << 20)

/** A draw that allocates nothing. It has no counterpart in kitrofimov/srp.
 *
 *  Arguments and result are those of srpDrawIndexBuffer (ib not NULL) or
 *  srpDrawVertexBuffer (ib NULL), computed by the same kernels. The ordinary
 *  draws grow their scratch buffers with cudaMalloc and cudaFree whenever a
 *  draw needs more than the draws before it. This one takes every scratch
 *  buffer from one array of SRP_GPU_FIXED_SCRATCH_BYTES in device memory
 *  that belongs to the library's device image, and calls no allocating
 *  routine. It is meant for callers that cannot have device memory allocated
 *  or freed in the middle of a frame: cudaFree waits for all work on the
 *  device, which stalls a renderer whose other streams must keep running,
 *  and a program that has given the rest of device memory to a caching
 *  allocator or to other processes may see a mid-frame allocation fail.
 *
 *  The first call on a device looks up the array's address (with that device
 *  current; the lookup loads the part of the library's device image that
 *  holds the array) and keeps it for later calls. No call may be made while
 *  the library's stream is being captured into a CUDA graph: partway through
 *  the draw the host waits for the counters of its setup stage, so such a
 *  call is rejected (-1 and a message) before anything is queued. Vertex and
 *  index buffers must already be in device memory, as
 *  srpVertexBufferCopyData / srpIndexBufferCopyData leave them when a GPU is
 *  present; the draw waits for copies queued by the Async variants.
 *
 *  Learned shading (srpGpuSetLearnedShading) and fragment capture
 *  (srpGpuMlpCapture) do not apply to these draws: they always run the
 *  program's own fragment shader, as if neither were set.
 *
 *  Limits. The parts of the scratch sized by the vertex buffer (about 64
 *  bytes and 4 per varying word per vertex), by the primitives (up to 96
 *  bytes each) and by the framebuffer (about 4 bytes per pixel) must leave at
 *  least 4 MiB of the array free; this is checked before anything runs. What
 *  the draw produces is checked once the setup stage has counted it: tile
 *  entries (about 16 bytes each) in three quarters of what is left,
 *  barycentric tables of large triangles in the other quarter, at most 16384
 *  vertices created by clipping and 4096 triangles that need clipping (whose
 *  extra triangles are counted in the primitive part). A line draw's entries
 *  are runs of up to 15 fragments in one tile, about one per tile a line
 *  crosses (one per step for lines that leave the framebuffer), at about
 *  340 bytes each with their fragment records.
 *  A draw beyond a limit is rejected: it returns -1, says which size was too
 *  large through the message callback and leaves the framebuffer unchanged.
 *
 *  Every call uses the same array. Each call clears, on the library's
 *  stream, the parts that must start at zero (counters, look-back flags,
 *  tile ranges, sort histograms) before using them, so calls in sequence on
 *  one stream are independent. Calls that overlap on the GPU (issued on
 *  different streams, or from several host threads) race on the array and
 *  give wrong images. Fragments of these draws are not added to the
 *  srpGpuGetStats fragment count, and stage profiling does not time them.
 *
 *  Returns 0 when the draw ran or had nothing to draw, -1 when it was
 *  rejected or a CUDA call failed. */
int srpGpuDrawFixedScratch(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                           const SRPShaderProgram* sp, SRPPrimitive prim, size_t startIndex, size_t count);

/* ------------------------------------------------------ stream, stats */

/** Launch all work on `stream` (a cudaStream_t; NULL = the library's own
 *  stream). Must be called outside of any draw. */
void srpGpuSetStream(void* stream);
void* srpGpuGetStream(void);
/** Block until all queued work has finished; reports pending device errors
 *  through the message callback. Returns 0 if no error was pending. */
int srpGpuSynchronize(void);

typedef struct SRPGpuStats
{
	uint64_t fragments;          /* fragments that passed coverage + scissor */
	uint64_t primitives;         /* primitives after clipping and culling */
	uint64_t binEntries;         /* (tile, primitive) pairs binned */
	uint64_t clipOverflows;      /* clipped polygons with more than 6 vertices */
	uint64_t draws;
	uint64_t kernelLaunches;     /* kernels launched by the library */
	uint64_t drawRetries;        /* draws run again after their scratch buffers grew */
} SRPGpuStats;

/** Read the counters accumulated since the last reset (waits for the GPU). */
void srpGpuGetStats(SRPGpuStats* stats);
void srpGpuResetStats(void);

/** Tile edge in pixels used by the binning and raster stages (8 or 16). */
void srpGpuSetTileSize(int tileSize);

/** Parts of a single draw (into a framebuffer whose width is a multiple of
 *  4) whose 8 x 8 framebuffer tiles move between global and shared memory by
 *  2-D tensor copies of the tensor-memory-access unit (TMA): */
#define SRP_GPU_TILE_COPY_RESOLVE_LOAD  1u  /* the light-tile resolve loads its depth tile */
#define SRP_GPU_TILE_COPY_RESOLVE_STORE 2u  /* and stores its depth and winning-fragment tiles */
#define SRP_GPU_TILE_COPY_SHADE         4u  /* the shading loads, updates and stores its colour tile */
/** Select them (0, the default: every kernel reads and writes the pixels
 *  directly). The images are the same whatever the selection. */
void srpGpuSetTileCopies(unsigned parts);

/* ----------------------------------------- failure-detection tests */

/* Every wait of a kernel on another block or on the tensor cores (the
 * look-back of the ordered setup, the mbarrier waits of learned shading) is
 * bounded: when it runs out, the kernel records a timeout, the draw stops or
 * falls back, and the error is reported through the message callback. These
 * calls make that path run, for tests; none has a counterpart in the
 * reference. */

/** Polls after which a bounded device wait gives up, for the draws issued
 *  from now on; 0 restores the default (2^24). */
void srpGpuSetWaitLimit(uint32_t iterations);

#define SRP_GPU_WAIT_TEST_SETUP   1u  /* the ordered setup's first block never publishes its prefix: the
                                         draw reports "Ordered-compaction wait timed out" and draws nothing */
#define SRP_GPU_WAIT_TEST_LEARNED 2u  /* learned shading issues no MMAs for its second layer: the draw
                                         reports the timeout and is shaded again by its own shader */
/** Withhold the selected signals (SRP_GPU_WAIT_TEST_*) from the draws issued
 *  from now on, so that the waits depending on them run out; 0 turns it off.
 *  Combine with a small srpGpuSetWaitLimit to keep the wait short. */
void srpGpuSetWaitTest(uint32_t flags);

/** The estimate of (tile, primitive) pairs per input primitive with which
 *  the next draw of each kind sizes its pair buffers; each draw replaces it
 *  with what it counted. A draw whose pairs exceed the estimate stops before
 *  its resolve, grows the buffers and runs again (srpGpuStats.drawRetries);
 *  0 forces that path on the next draw. */
void srpGpuSetEntryEstimate(double entriesPerPrimitive);

/* ---------------------------------------------------------- profiling */

typedef enum SRPGpuStage
{
	SRP_GPU_STAGE_VERTEX = 0,   /* index range + vertex shading */
	SRP_GPU_STAGE_SETUP,        /* assembly, clipping, setup, ordered compaction */
	SRP_GPU_STAGE_BIN,          /* big-primitive pairs, lambda tables, line DDA, sort */
	SRP_GPU_STAGE_RESOLVE,      /* per-tile coverage, stencil and depth */
	SRP_GPU_STAGE_SHADE,        /* deferred fragment shading */
	SRP_GPU_STAGE_COUNT
} SRPGpuStage;

typedef struct SRPGpuProfile
{
	double ms[SRP_GPU_STAGE_COUNT];        /* device time per stage (CUDA events) */
	uint64_t launches[SRP_GPU_STAGE_COUNT];
	uint64_t resolveTiles;                 /* tiles handled by the resolve stage */
	uint64_t resolveItems;                 /* (tile, item) pairs it consumed */
} SRPGpuProfile;

/** Replay repeated draws from CUDA graphs (on by default). A draw's work
 *  after its host-side preparation is captured once per distinct set of
 *  draw parameters and launch sizes, and relaunched as graphs, one per
 *  sequence of the draw on each of its streams, when the same draw comes
 *  again (the host reads the draw's counters between them).
 *  Stage profiling launches directly. */
void srpGpuSetDrawGraphs(int enable);
/** Overlap of consecutive draws (default on): a draw's vertex, setup and
 *  binning stages run on a front stream of the library (one per scratch set,
 *  the sets alternating between draws), beside the previous draw's front,
 *  resolve and shading, and its resolve on another stream, beside the
 *  previous draw's shading. Resolves stay in submission order among
 *  themselves, and so do shadings, which run on the library's stream.
 *  Results are identical either way. */
void srpGpuSetDrawOverlap(int enable);

/** Record CUDA events around every stage of every draw (off by default). */
void srpGpuSetProfiling(int enable);
/** Sum of the recorded stage times since the last reset (waits for the GPU). */
void srpGpuGetProfile(SRPGpuProfile* profile);
void srpGpuResetProfile(void);

#ifdef __cplusplus
}
#endif
