/* srp-gb300: the built-in shader library, shared by host and device.
 *
 * The reference (kitrofimov/srp, include/srp/shaders.h:44-86) takes shaders as
 * host function pointers, which a GPU cannot call. This library therefore
 * ships its shaders as source in srp/shaderlib_impl.h, written once and
 * compiled both as host C (the functions declared below, exported by every
 * build of the library) and as __device__ code inside the GPU kernels. Passing
 * one of the functions below as SRPVertexShader.shader / SRPFragmentShader.shader
 * selects the matching device shader; other host functions must be mapped with
 * srpGpuRegisterVertexShader / srpGpuRegisterFragmentShader (srp/gpu.h).
 *
 * Every built-in shader reads the same uniform block, SRPStdUniform. */
#pragma once

#include <stdint.h>
#include "srp/shaders.h"
#include "srp/mat.h"
#include "srp/texture.h"

#define SRP_STD_MAX_LIGHTS 16
#define SRP_STD_MAX_PASS   16

/** Packed mixed-type varying block read by srpFsMixed, at byte
 *  4*varyingOffset: +0 int8, +1 double[2], +17 uint16, +19 float[2],
 *  +27 int16, +29 uint64 (37 bytes, every member but the first unaligned). */
#define SRP_MIXED_BLOCK_BYTES 37

/** Uniform block read by all built-in shaders. Vertex layouts are described
 *  in 32-bit words: the position is always words 0..2 of the vertex. */
typedef struct SRPStdUniform
{
	mat4 model;
	mat4 view;
	mat4 projection;
	float color[4];          /* solid colour / tint */
	float cameraPos[4];      /* world-space eye position (lighting shaders) */
	float lightPos[SRP_STD_MAX_LIGHTS][4];    /* xyz + unused */
	float lightColor[SRP_STD_MAX_LIGHTS][4];  /* rgb + unused */
	float ambient[4];
	float shininess;
	float marbleFrequency;   /* srpFsMarble base frequency */
	float marbleGain;        /* srpFsMarble per-octave gain */
	float depthScale;        /* srpFsDepthOverwrite: fragDepth = z * scale + bias */
	float depthBias;
	uint32_t nLights;
	uint32_t marbleOctaves;
	uint32_t passOffset;     /* srpVsTransform: first vertex word copied to varyings;
	                            srpVsBytes: first vertex byte (< 64) */
	uint32_t passCount;      /* srpVsTransform: number of words copied (<= 16);
	                            srpVsBytes: number of bytes copied (<= 64) */
	uint32_t normalOffset;   /* srpVsWorld: vertex word offset of the normal */
	uint32_t uvOffset;       /* srpVsWorld: vertex word offset of the uv */
	uint32_t extraOffset;    /* srpVsWorld: first extra word appended to varyings */
	uint32_t extraCount;     /* srpVsWorld: number of extra words (<= 16) */
	uint32_t varyingOffset;  /* fragment shaders: first varying word they read */
	float texelScale;        /* srpFsTextureLod: texels per pixel at clip w = 1 */
	SRPTexture* texture;     /* replaced by a device descriptor on upload */
} SRPStdUniform;

/** Device shader identifiers (see srp/gpu.h for the mapping API). */
typedef enum SRPGpuVertexShaderId
{
	SRP_GPU_VS_NONE = 0,
	SRP_GPU_VS_TRANSFORM = 1,  /* clip = P*(V*(M*pos)); varyings = passthrough words */
	SRP_GPU_VS_WORLD = 2,      /* varyings = world pos, world normal, uv, extras */
	SRP_GPU_VS_BYTES = 3,      /* clip as TRANSFORM; varyings = passCount raw vertex bytes from byte passOffset */
	SRP_GPU_VS_COUNT
} SRPGpuVertexShaderId;

typedef enum SRPGpuFragmentShaderId
{
	SRP_GPU_FS_NONE = 0,
	SRP_GPU_FS_VARYING_COLOR = 1,   /* rgb = varyings[o..o+2] */
	SRP_GPU_FS_SOLID = 2,           /* rgba = uniform colour */
	SRP_GPU_FS_PRIMITIVE_ID = 3,    /* colour hashed from primitiveID */
	SRP_GPU_FS_TEXTURE = 4,         /* texture(uv = varyings[o..o+1]) */
	SRP_GPU_FS_TEXTURE_MODULATE = 5,/* texture(uv) * colour(o+2..o+4) * tint(flat u32 at o+5) */
	SRP_GPU_FS_BLINN_PHONG = 6,     /* textured Blinn-Phong from srpVsWorld varyings */
	SRP_GPU_FS_MARBLE = 7,          /* value-noise marble + point lights (expensive) */
	SRP_GPU_FS_DEPTH_OVERWRITE = 8, /* colour from varyings, writes fragDepth (late Z) */
	SRP_GPU_FS_FRAGCOORD = 9,       /* colour from fragCoord and frontFacing */
	SRP_GPU_FS_FLAT_INT = 10,       /* palette colour from an int32 varying at word o */
	SRP_GPU_FS_MIXED = 11,          /* colour from the packed mixed-type block at word o (srpFsMixed) */
	SRP_GPU_FS_BYTE_PALETTE = 12,   /* 0 red, 1 green, 2 blue, else hashed: uint8 varying at byte 4*o */
	SRP_GPU_FS_PRIMITIVE_MOD = 13,  /* ((id*97, id*57, id*23) mod 255) / 255 / colour[0] */
	SRP_GPU_FS_TEXTURE_LOD = 14,    /* texture(uv = varyings[o..o+1]) at lod log2(max(1, texelScale * w)) */
	SRP_GPU_FS_COUNT
} SRPGpuFragmentShaderId;

#ifdef __cplusplus
extern "C" {
#endif

/* Host entry points of the built-in shaders. */
void srpVsTransform(SRPVertexShaderIn* in, SRPVertexShaderOut* out);
void srpVsWorld(SRPVertexShaderIn* in, SRPVertexShaderOut* out);
void srpVsBytes(SRPVertexShaderIn* in, SRPVertexShaderOut* out);
void srpFsVaryingColor(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsSolid(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsPrimitiveId(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsTexture(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsTextureModulate(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsBlinnPhong(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsMarble(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsDepthOverwrite(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsFragCoord(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsFlatInt(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsMixed(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsBytePalette(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsPrimitiveMod(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);
void srpFsTextureLod(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out);

#ifdef __cplusplus
}
#endif
