/* srp-gb300 public API: vertex and index buffers and the draw calls.
 *
 * Replaces include/srp/buffer.h of kitrofimov/srp (buffer.h:18-92).
 * CopyData stores the bytes in a host staging copy (as the reference's memcpy
 * does); the upload to HBM happens once, at the next draw that uses the
 * buffer. Draws run on the GPU; errors (out-of-range draw, unknown primitive,
 * unmapped shader, CUDA failure) are reported through the message callback. */
#pragma once

#include "srp/framebuffer.h"
#include "srp/shaders.h"

typedef enum SRPPrimitive
{
	SRP_PRIM_POINTS,
	SRP_PRIM_LINES,           /* odd trailing vertex ignored */
	SRP_PRIM_LINE_STRIP,
	SRP_PRIM_LINE_LOOP,
	SRP_PRIM_TRIANGLES,
	SRP_PRIM_TRIANGLE_STRIP,  /* odd triangles swap their first two vertices */
	SRP_PRIM_TRIANGLE_FAN
} SRPPrimitive;

typedef struct SRPVertexBuffer SRPVertexBuffer;
typedef struct SRPIndexBuffer SRPIndexBuffer;

#ifdef __cplusplus
extern "C" {
#endif

SRPVertexBuffer* srpNewVertexBuffer(void);                                    /* buffer.h:38 */
void srpFreeVertexBuffer(SRPVertexBuffer* vb);                                /* buffer.h:42 */
void srpVertexBufferCopyData(SRPVertexBuffer* vb, size_t nBytesPerVertex,
                             size_t nBytesData, const void* data);            /* buffer.h:49-50 */
void srpDrawVertexBuffer(const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                         const SRPShaderProgram* sp, SRPPrimitive primitive,
                         size_t startIndex, size_t count);                    /* buffer.h:59-62 */

SRPIndexBuffer* srpNewIndexBuffer(void);                                      /* buffer.h:66 */
/* indicesType must be SRP_UINT8, SRP_UINT16, SRP_UINT32 or SRP_UINT64. */
void srpIndexBufferCopyData(SRPIndexBuffer* ib, SRPType indicesType,
                            size_t nBytesData, const void* data);             /* buffer.h:74-75 */
void srpFreeIndexBuffer(SRPIndexBuffer* ib);                                  /* buffer.h:79 */
void srpDrawIndexBuffer(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb,
                        const SRPFramebuffer* fb, const SRPShaderProgram* sp,
                        SRPPrimitive primitive, size_t startIndex, size_t count); /* buffer.h:89-92 */

#ifdef __cplusplus
}
#endif
