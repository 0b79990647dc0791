/* Host-side pieces of a draw that srp_fixed.cu (the fixed-scratch draw)
 * takes from srp_api.cu. None of these functions allocates memory, on the
 * host or on the device. */
#pragma once

#include <cuda_runtime.h>
#include "srp/srp.h"
#include "kernels.h"

namespace srpg {

/* Width of the radix-sort key for tile numbers below n, in whole 8-bit
 * digits: the ordinary and the fixed-scratch draw sort with the same key, so
 * that their per-tile item orders, and therefore their images, are equal. */
inline uint32_t sortKeyBits(uint32_t n)
{
	uint32_t b = 0;
	while ((1ull << b) < (unsigned long long) n + 1ull) ++b;
	return (b + 7) / 8 * 8;
}

struct FixedDrawInfo {
	cudaStream_t stream;   /* the library's stream */
	size_t nIn;            /* input primitives of the draw */
	size_t outPer;         /* primitives emitted per input primitive (3 for wireframe/point triangles) */
	uint32_t numTiles;     /* 8x8 tiles of the framebuffer */
	size_t pixels;         /* framebuffer pixels */
	int kind;              /* kKindTri, kKindLineFrag or kKindPoint */
	bool triangles;        /* a triangle primitive: the clip pre-pass runs */
	bool late;             /* the fragment shader writes depth: late-depth resolve */
	bool coherent;         /* SRP_GPU_FB_COHERENT: host planes mirrored around the draw */
};

/* Validates a draw exactly as srpDrawIndexBuffer / srpDrawVertexBuffer do and
 * fills every field of P that does not point into scratch memory (state
 * snapshot, varying layout, uniform, shader ids, buffers, framebuffer
 * planes). Rejects, with a message, what the ordinary draw would only handle
 * by allocating: a buffer whose bytes are not in device memory yet, a texture
 * without device texels, an uninitialised library.
 * Returns 0 when the draw is ready, 1 when there is nothing to draw, -1 when
 * it was rejected. */
int fixedDrawPrepare(DrawParams& P, const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                     const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count, FixedDrawInfo& info);

/* Reports an error through the user's message callback. */
void fixedDrawError(const char* fn, const char* fmt, ...);

/* Copies the host planes to the device planes, or back (and waits). */
void fixedDrawUpload(const SRPFramebuffer* fb);
void fixedDrawDownload(const SRPFramebuffer* fb);

/* Adds a finished draw's counters to the statistics of srpGpuGetStats. */
void fixedDrawAccount(const DeviceCounters& c, unsigned launches);

}  // namespace srpg
