/* srp-gb300 public API: framebuffer.
 *
 * Replaces include/srp/framebuffer.h of kitrofimov/srp (framebuffer.h:17-39).
 * The struct layout is identical; `color`, `depth` and `stencil` are HOST
 * mirrors (pinned memory) of the device-resident planes the GPU draws into.
 * See srp/gpu.h for when the mirrors are refreshed. */
#pragma once

#include <stddef.h>
#include <stdint.h>

/** A W x H colour (packed RGBA8), fp32 depth and 8-bit stencil framebuffer,
 *  row-major, pixel (x, y) at index y * width + x. */
typedef struct SRPFramebuffer
{
	size_t width;
	size_t height;
	size_t size;        /* width * height */
	uint32_t* color;
	float* depth;
	uint8_t* stencil;
} SRPFramebuffer;

#ifdef __cplusplus
extern "C" {
#endif

/** Create a framebuffer (replaces framebuffer.h:31). Stencil starts at 0. */
SRPFramebuffer* srpNewFramebuffer(size_t width, size_t height);

/** Destroy a framebuffer created by srpNewFramebuffer (framebuffer.h:35). */
void srpFreeFramebuffer(SRPFramebuffer* fb);

/** Set colour to 0 and depth to -1; stencil is left as it is
 *  (framebuffer.h:39, semantics of src/core/framebuffer.c:57-62). */
void srpFramebufferClear(const SRPFramebuffer* fb);

#ifdef __cplusplus
}
#endif
