/* Seeded synthetic scenes driven through the public srp API.
 *
 * The same source is compiled against three implementations of the API: the
 * GPU library (SCENES_GPU), the CPU oracle, and the reference library built
 * from source (SCENES_REF). Inputs are generated with integer PRNG draws and
 * double arithmetic only (no libm transcendental calls, no contraction), so a
 * given (scene, seed, scale) produces bit-identical vertex, index and uniform
 * bytes on x86-64 and AArch64; sceneInputHash() checks that. */
#pragma once

#include <stddef.h>
#include <stdint.h>
#include "srp/srp.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct Scene Scene;

typedef struct SceneInfo {
	int width, height;
	size_t inputTriangles, inputLines, inputPoints;   /* primitives submitted per frame */
	size_t vertexBytes, indexBytes, textureBytes;    /* per-frame input bytes */
	int draws;                                       /* draw calls per frame */
	int usesStencil;
} SceneInfo;

/* Names of all scenes, NULL-terminated. */
const char* const* sceneNames(void);

/* Build scene `name` (seed, size scale in (0, 1]; 1 = full size). Creates the
 * srp buffers, textures and shader programs. NULL if the name is unknown. */
Scene* sceneCreate(const char* name, uint64_t seed, double scale);
void sceneDestroy(Scene* s);
void sceneGetInfo(const Scene* s, SceneInfo* info);
uint64_t sceneInputHash(const Scene* s);

/* Copy the host vertex/index data into the srp buffers again
 * (srpVertexBufferCopyData / srpIndexBufferCopyData), as a frame whose
 * geometry comes from host memory would. */
void sceneUpload(Scene* s);

/* Clear the framebuffer and set the scene's initial depth and stencil. */
void scenePrepareFramebuffer(Scene* s, SRPFramebuffer* fb);

/* Set the pipeline state and issue the scene's draw calls. */
void sceneRender(Scene* s, SRPFramebuffer* fb);

/* Write the scene's generated inputs (vertex, index, texture and uniform
 * bytes, pointer fields excluded) to `path`; used to compare machines. */
int sceneDumpInputs(const Scene* s, const char* path);

#ifdef SCENES_GPU
#include "srp/gpu.h"
/* Batched workload ("bscene" scenes, one draw each): the scene's draw as an
 * srpGpuDrawBatch entry (returns nonzero for other scenes), and one batched
 * render of n scenes into their framebuffers with the scenes' state. */
int sceneDrawDesc(Scene* s, SRPFramebuffer* fb, SRPGpuDraw* out);
void sceneBatchRender(Scene** scenes, SRPFramebuffer** fbs, size_t n, SRPGpuDraw* scratch);
/* srpGpuAutotune on that batch (the framebuffers must be prepared again). */
int sceneBatchAutotune(Scene** scenes, SRPFramebuffer** fbs, size_t n, SRPGpuDraw* scratch, int repeats,
                       SRPGpuTuning* best);
/* sceneUpload with the asynchronous copies (srpGpu*CopyDataAsync): the
 * scene's host data must stay unchanged until srpGpuSynchronize. */
void sceneUploadAsync(Scene* s);
/* sceneUploadAsync of n scenes with the Batch copies, 256 scenes at a time
 * (their vertex buffers, then their index buffers), so that the first
 * scenes' buffers arrive first. */
void sceneUploadBatchAsync(Scene** scenes, size_t n);
/* scenePrepareFramebuffer of n scenes in one srpGpuFramebufferFillBatch when
 * they share their initial depth and stencil (else one by one). */
void scenePrepareBatch(Scene** scenes, SRPFramebuffer** fbs, size_t n);
/* Draw every scene through srpGpuDrawFixedScratch (on) or the ordinary draw
 * calls (off, the default); the count of fixed-scratch draws rejected since
 * the switch was last set. */
void sceneUseFixedScratch(int on);
int sceneFixedScratchRejected(void);
#endif

/* Convenience: create a framebuffer of the scene's size, prepare, render, copy
 * the planes out (color W*H u32, depth W*H f32, stencil W*H u8). Returns 0 on
 * success. */
int sceneRunOnce(const char* name, uint64_t seed, double scale,
                 uint32_t* color, float* depth, uint8_t* stencil, int* width, int* height);

#ifdef __cplusplus
}
#endif
