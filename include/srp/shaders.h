/* srp-gb300 public API: shader program types.
 *
 * Replaces include/srp/shaders.h of kitrofimov/srp (shaders.h:24-97); struct
 * layouts are identical. A GPU cannot call host function pointers, so the
 * `shader` members are used as keys: srp/gpu.h maps each host function to a
 * device shader compiled from the shared header srp/shaderlib_impl.h. Drawing
 * with an unmapped shader is an error reported through the message callback
 * (there is no CPU fallback). */
#pragma once

#include <stdbool.h>
#include <stddef.h>
#include "srp/vertex.h"

/** User uniform block (opaque). */
typedef struct SRPUniform SRPUniform;

/** Vertex shader inputs. */
typedef struct SRPVertexShaderIn
{
	SRPUniform* uniform;
	SRPVertex* vertex;
	size_t vertexID;
} SRPVertexShaderIn;

/** Vertex shader outputs: clip-space position (NDC after the divide) and a
 *  pointer to this vertex's varying block. */
typedef struct SRPVertexShaderOut
{
	union {
		float clipPosition[4];
		float ndcPosition[4];
	};
	SRPVarying* varyings;
} SRPVertexShaderOut;

typedef struct SRPVertexShader
{
	void (*shader)(SRPVertexShaderIn* in, SRPVertexShaderOut* out);
	size_t nVaryings;
	SRPVaryingInfo* varyingsInfo;
	size_t varyingsSize;
} SRPVertexShader;

/** Fragment shader inputs. fragCoord = (x + 0.5, y + 0.5, depth, 1/w). */
typedef struct SRPFragmentShaderIn
{
	SRPUniform* uniform;
	SRPInterpolated* varyings;
	float fragCoord[4];
	bool frontFacing;
	size_t primitiveID;
} SRPFragmentShaderIn;

/** Fragment shader outputs; fragDepth is honoured only when the shader is
 *  declared with mayOverwriteDepth = true and it is not NaN. */
typedef struct SRPFragmentShaderOut
{
	float color[4];
	float fragDepth;
} SRPFragmentShaderOut;

typedef struct SRPFragmentShader
{
	void (*shader)(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
	bool mayOverwriteDepth;
} SRPFragmentShader;

/** Uniform + vertex shader + fragment shader used by one draw. */
typedef struct SRPShaderProgram
{
	SRPUniform* uniform;
	SRPVertexShader* vs;
	SRPFragmentShader* fs;
} SRPShaderProgram;
