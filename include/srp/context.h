/* srp-gb300 public API: global pipeline state.
 *
 * Replaces include/srp/context.h of kitrofimov/srp (context.h:20-194). The
 * struct layout and the defaults set by srpNewContext are identical, including
 * the reference's quirks (depth compare defaults to GREATER; srpStencilTest
 * enables the test whatever its argument). As in the reference, the user
 * program defines the global `SRPContext srpContext;` and initialises it with
 * srpNewContext(&srpContext). */
#pragma once

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include "srp/message_callback.h"
#include "srp/arena.h"

typedef enum SRPProvokingVertexMode
{
	SRP_PROVOKING_VERTEX_FIRST,
	SRP_PROVOKING_VERTEX_LAST
} SRPProvokingVertexMode;

typedef enum SRPWinding
{
	SRP_WINDING_CCW,
	SRP_WINDING_CW
} SRPWinding;

typedef enum SRPFace
{
	SRP_FACE_NONE,
	SRP_FACE_FRONT,
	SRP_FACE_BACK,
	SRP_FACE_FRONT_AND_BACK
} SRPFace;

typedef enum SRPPolygonMode
{
	SRP_POLYGON_MODE_FILL,
	SRP_POLYGON_MODE_LINE,
	SRP_POLYGON_MODE_POINT
} SRPPolygonMode;

typedef enum SRPCompareOp
{
	SRP_COMPARE_NEVER,
	SRP_COMPARE_ALWAYS,
	SRP_COMPARE_LESS,
	SRP_COMPARE_LEQUAL,
	SRP_COMPARE_GREATER,
	SRP_COMPARE_GEQUAL,
	SRP_COMPARE_EQUAL,
	SRP_COMPARE_NOTEQUAL
} SRPCompareOp;

typedef enum {
	SRP_STENCIL_KEEP,
	SRP_STENCIL_ZERO,
	SRP_STENCIL_REPLACE,
	SRP_STENCIL_INCR,       /* saturates at 255 */
	SRP_STENCIL_INCR_WRAP,
	SRP_STENCIL_DECR,       /* saturates at 0 */
	SRP_STENCIL_DECR_WRAP,
	SRP_STENCIL_INVERT
} SRPStencilOp;

typedef struct SRPRasterState
{
	SRPWinding frontFace;
	SRPFace cullFace;
	SRPPolygonMode polygonMode;
	float pointSize;
} SRPRasterState;

/** Scissor box: pixels with x0 <= x < x0 + width and y0 <= y < y0 + height
 *  pass when enabled. */
typedef struct SRPScissorState {
	bool enabled;
	size_t x;
	size_t y;
	size_t width;
	size_t height;
} SRPScissorState;

/** Per-face stencil state: compare (ref & mask) OP (stored & mask); updates
 *  are written through writeMask. */
typedef struct SRPStencilFaceState {
	SRPCompareOp func;
	uint8_t ref;
	uint8_t mask;
	uint8_t writeMask;
	SRPStencilOp sfailOp;
	SRPStencilOp dfailOp;
	SRPStencilOp passOp;
} SRPStencilFaceState;

typedef struct SRPStencilState {
	bool enabled;
	SRPStencilFaceState front;
	SRPStencilFaceState back;
} SRPStencilState;

/** Depth state; depth is written only when both testEnable and writeEnable
 *  are set. */
typedef struct SRPDepthState
{
	bool testEnable;
	bool writeEnable;
	SRPCompareOp compareOp;
} SRPDepthState;

typedef struct SRPContext
{
	SRPMessageCallback messageCallback;
	SRPProvokingVertexMode provokingVertexMode;
	SRPRasterState raster;
	SRPScissorState scissor;
	SRPStencilState stencil;
	SRPDepthState depth;
	SRPArena* arena;
} SRPContext;

#ifdef __cplusplus
extern "C" {
#endif

/* Each setter replaces the declaration at the cited line of the reference's
 * include/srp/context.h. */
void srpNewContext(SRPContext* pContext);                                   /* context.h:148 */
void srpSetMessageCallback(SRPMessageCallback callback);                    /* context.h:151 */
void srpProvokingVertexMode(SRPProvokingVertexMode mode);                   /* context.h:154 */
void srpRasterCullFace(SRPFace face);                                       /* context.h:157 */
void srpRasterFrontFace(SRPWinding face);                                   /* context.h:159 */
void srpRasterPolygonMode(SRPPolygonMode mode);                             /* context.h:161 */
void srpRasterPointSize(float size);                                        /* context.h:163 */
void srpScissorTest(bool enable);                                           /* context.h:166 */
void srpScissorOptions(size_t x, size_t y, size_t width, size_t height);    /* context.h:168 */
void srpStencilTest(bool enable);                                           /* context.h:171 */
void srpStencilFunc(SRPCompareOp func, uint8_t ref, uint8_t mask);          /* context.h:173 */
void srpStencilFuncSeparate(SRPFace face, SRPCompareOp func, uint8_t ref, uint8_t mask); /* context.h:175 */
void srpStencilOp(SRPStencilOp sfail, SRPStencilOp dfail, SRPStencilOp pass);            /* context.h:177 */
void srpStencilOpSeparate(SRPFace face, SRPStencilOp sfail, SRPStencilOp dfail, SRPStencilOp pass); /* context.h:179 */
void srpStencilWriteMask(uint8_t mask);                                     /* context.h:181 */
void srpStencilWriteMaskSeparate(SRPFace face, uint8_t mask);               /* context.h:183 */
void srpDepthTest(bool enable);                                             /* context.h:186 */
void srpDepthWrite(bool enable);                                            /* context.h:188 */
void srpDepthCompareOp(SRPCompareOp op);                                    /* context.h:190 */

/** The global context, defined by the user program (context.h:194). */
extern SRPContext srpContext;

#ifdef __cplusplus
}
#endif
