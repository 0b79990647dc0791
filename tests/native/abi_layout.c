/* Prints the size and member offsets of every public struct and union of
 * srp's C API, and the values of the last enumerator of each public enum.
 * Compiled once against this library's headers (include/) and once against
 * the reference's (include/ of kitrofimov/srp), the two outputs must be
 * identical: a program built against the reference then passes the same
 * bytes to this library (tests/test_abi.py). */
#define SRP_INCLUDE_VEC
#define SRP_INCLUDE_MAT
#include <stddef.h>
#include <stdio.h>
#include "srp/srp.h"

#define SIZE(T) printf("sizeof %s %zu align %zu\n", #T, sizeof(T), _Alignof(T))
#define OFF(T, m) printf("offsetof %s.%s %zu\n", #T, #m, offsetof(T, m))
#define ENUM(e) printf("enum %s %d\n", #e, (int) (e))

int main(void)
{
	SIZE(SRPContext);
	OFF(SRPContext, messageCallback); OFF(SRPContext, provokingVertexMode); OFF(SRPContext, raster);
	OFF(SRPContext, scissor); OFF(SRPContext, stencil); OFF(SRPContext, depth); OFF(SRPContext, arena);
	SIZE(SRPRasterState);
	OFF(SRPRasterState, frontFace); OFF(SRPRasterState, cullFace); OFF(SRPRasterState, polygonMode);
	OFF(SRPRasterState, pointSize);
	SIZE(SRPScissorState);
	OFF(SRPScissorState, enabled); OFF(SRPScissorState, x); OFF(SRPScissorState, y); OFF(SRPScissorState, width);
	OFF(SRPScissorState, height);
	SIZE(SRPStencilFaceState);
	OFF(SRPStencilFaceState, func); OFF(SRPStencilFaceState, ref); OFF(SRPStencilFaceState, mask);
	OFF(SRPStencilFaceState, writeMask); OFF(SRPStencilFaceState, sfailOp); OFF(SRPStencilFaceState, dfailOp);
	OFF(SRPStencilFaceState, passOp);
	SIZE(SRPStencilState);
	OFF(SRPStencilState, enabled); OFF(SRPStencilState, front); OFF(SRPStencilState, back);
	SIZE(SRPDepthState);
	OFF(SRPDepthState, testEnable); OFF(SRPDepthState, writeEnable); OFF(SRPDepthState, compareOp);
	SIZE(SRPMessageCallback);
	OFF(SRPMessageCallback, func); OFF(SRPMessageCallback, userParameter);
	SIZE(SRPVertexShaderIn);
	OFF(SRPVertexShaderIn, uniform); OFF(SRPVertexShaderIn, vertex); OFF(SRPVertexShaderIn, vertexID);
	SIZE(SRPVertexShaderOut);
	OFF(SRPVertexShaderOut, clipPosition); OFF(SRPVertexShaderOut, ndcPosition); OFF(SRPVertexShaderOut, varyings);
	SIZE(SRPVertexShader);
	OFF(SRPVertexShader, shader); OFF(SRPVertexShader, nVaryings); OFF(SRPVertexShader, varyingsInfo);
	OFF(SRPVertexShader, varyingsSize);
	SIZE(SRPFragmentShaderIn);
	OFF(SRPFragmentShaderIn, uniform); OFF(SRPFragmentShaderIn, varyings); OFF(SRPFragmentShaderIn, fragCoord);
	OFF(SRPFragmentShaderIn, frontFacing); OFF(SRPFragmentShaderIn, primitiveID);
	SIZE(SRPFragmentShaderOut);
	OFF(SRPFragmentShaderOut, color); OFF(SRPFragmentShaderOut, fragDepth);
	SIZE(SRPFragmentShader);
	OFF(SRPFragmentShader, shader); OFF(SRPFragmentShader, mayOverwriteDepth);
	SIZE(SRPShaderProgram);
	OFF(SRPShaderProgram, uniform); OFF(SRPShaderProgram, vs); OFF(SRPShaderProgram, fs);
	SIZE(SRPFramebuffer);
	OFF(SRPFramebuffer, width); OFF(SRPFramebuffer, height); OFF(SRPFramebuffer, size); OFF(SRPFramebuffer, color);
	OFF(SRPFramebuffer, depth); OFF(SRPFramebuffer, stencil);
	SIZE(SRPVaryingInfo);
	OFF(SRPVaryingInfo, nItems); OFF(SRPVaryingInfo, type); OFF(SRPVaryingInfo, interpolationMode);
	SIZE(SRPColor);
	SIZE(vec2); SIZE(vec3); SIZE(vec4); SIZE(mat4);
	SIZE(SRPPrimitive); SIZE(SRPType); SIZE(SRPCompareOp); SIZE(SRPStencilOp);
	ENUM(SRP_PRIM_TRIANGLE_FAN); ENUM(SRP_UINT64); ENUM(SRP_COMPARE_NOTEQUAL); ENUM(SRP_STENCIL_INVERT);
	ENUM(SRP_POLYGON_MODE_POINT); ENUM(SRP_FACE_FRONT_AND_BACK); ENUM(SRP_WINDING_CW);
	ENUM(SRP_PROVOKING_VERTEX_LAST); ENUM(SRP_INTERPOLATION_MODE_FLAT); ENUM(TW_CLAMP_TO_EDGE);
	ENUM(SRP_MESSAGE_SEVERITY_HIGH); ENUM(SRP_MESSAGE_ERROR);
	return 0;
}
