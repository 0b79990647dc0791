/* srp-gb300: bodies of the built-in shaders, written once for host and device.
 *
 * This header is included (a) by host C code, which wraps each body in the
 * exported functions declared in srp/shaderlib.h, and (b) by the CUDA kernels,
 * which call the bodies as __device__ functions. The including translation
 * unit must compile without floating-point contraction (gcc -ffp-contract=off,
 * nvcc -fmad=false): the vertex transform feeds coverage and depth and has to
 * round exactly like the reference's mat4MultiplyVec4 (src/math/mat.c:16-45).
 *
 * Device builds define SRP_DEVICE_TEXTURE_SAMPLE(tex, u, v, out) and
 * SRP_DEVICE_TEXTURE_SAMPLE_LOD(tex, u, v, lod, out) before including this
 * header; the host build calls srpTextureGetFilteredColor(Lod). */
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>
#include "srp/shaderlib.h"

#if defined(__CUDACC__) && !defined(SRP_SHADERLIB_HOST_ONLY)
#define SRP_SHADER_FN static inline __host__ __device__
#else
#define SRP_SHADER_FN static inline
#endif

#if defined(__CUDA_ARCH__) && !defined(SRP_SHADERLIB_HOST_ONLY)
#define SRP_TEXTURE_SAMPLE(tex, u, v, out) SRP_DEVICE_TEXTURE_SAMPLE(tex, u, v, out)
#define SRP_TEXTURE_SAMPLE_LOD(tex, u, v, lod, out) SRP_DEVICE_TEXTURE_SAMPLE_LOD(tex, u, v, lod, out)
#elif defined(SRP_SHADERLIB_NEAREST_ONLY)
/* host build linked against a library without the filtering additions of
 * srp/texture.h (the reference's own): every sample is at level 0 */
#define SRP_TEXTURE_SAMPLE(tex, u, v, out) srpTextureGetFilteredColor(tex, u, v, out)
#define SRP_TEXTURE_SAMPLE_LOD(tex, u, v, lod, out) srpTextureGetFilteredColor(tex, u, v, out)
#else
#define SRP_TEXTURE_SAMPLE(tex, u, v, out) srpTextureGetFilteredColor(tex, u, v, out)
#define SRP_TEXTURE_SAMPLE_LOD(tex, u, v, lod, out) srpTextureGetFilteredColorLod(tex, u, v, lod, out)
#endif

/* Word access through memcpy: user vertex and varying blocks may be byte
 * packed on the host; on the device they live in aligned local arrays. */
SRP_SHADER_FN float srpslLoadF(const void* base, uint32_t word)
{
	float f;
	memcpy(&f, (const unsigned char*) base + 4u * word, 4);
	return f;
}

SRP_SHADER_FN uint32_t srpslLoadU(const void* base, uint32_t word)
{
	uint32_t u;
	memcpy(&u, (const unsigned char*) base + 4u * word, 4);
	return u;
}

SRP_SHADER_FN void srpslStoreU(void* base, uint32_t word, uint32_t value)
{
	memcpy((unsigned char*) base + 4u * word, &value, 4);
}

SRP_SHADER_FN void srpslStoreF(void* base, uint32_t word, float value)
{
	memcpy((unsigned char*) base + 4u * word, &value, 4);
}

/* r = m * v with each row summed left to right: ((a*x + b*y) + c*z) + d*w. */
SRP_SHADER_FN void srpslMatVec(const mat4* m, const float v[4], float r[4])
{
	for (int i = 0; i < 4; ++i)
		r[i] = m->data[i][0] * v[0] + m->data[i][1] * v[1] + m->data[i][2] * v[2] + m->data[i][3] * v[3];
}

SRP_SHADER_FN float srpslDot3(const float a[3], const float b[3])
{
	return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

SRP_SHADER_FN void srpslNormalize3(float v[3])
{
	float len = sqrtf(srpslDot3(v, v));
	float inv = (len > 0.0f) ? 1.0f / len : 0.0f;
	v[0] *= inv; v[1] *= inv; v[2] *= inv;
}

SRP_SHADER_FN float srpslClamp01(float x)
{
	return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
}

/* ---------------------------------------------------------------- vertex */

/* Position at words 0..2, clip = P * (V * (M * (pos, 1))), then `passCount`
 * words starting at `passOffset` are copied to the varyings unchanged. */
SRP_SHADER_FN void srpslVsTransform(SRPVertexShaderIn* in, SRPVertexShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	const void* vtx = (const void*) in->vertex;
	float p[4] = { srpslLoadF(vtx, 0), srpslLoadF(vtx, 1), srpslLoadF(vtx, 2), 1.0f };
	float a[4], b[4];
	srpslMatVec(&u->model, p, a);
	srpslMatVec(&u->view, a, b);
	srpslMatVec(&u->projection, b, out->clipPosition);
	for (uint32_t w = 0; w < SRP_STD_MAX_PASS; ++w)
		if (w < u->passCount)
			srpslStoreU(out->varyings, w, srpslLoadU(vtx, u->passOffset + w));
}

/* Varyings: world position (3), world normal (3), uv (2), then `extraCount`
 * words starting at vertex word `extraOffset`. */
SRP_SHADER_FN void srpslVsWorld(SRPVertexShaderIn* in, SRPVertexShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	const void* vtx = (const void*) in->vertex;
	float p[4] = { srpslLoadF(vtx, 0), srpslLoadF(vtx, 1), srpslLoadF(vtx, 2), 1.0f };
	float n[4] = { srpslLoadF(vtx, u->normalOffset), srpslLoadF(vtx, u->normalOffset + 1),
	               srpslLoadF(vtx, u->normalOffset + 2), 0.0f };
	float world[4], wn[4], view[4];
	srpslMatVec(&u->model, p, world);
	srpslMatVec(&u->model, n, wn);
	srpslMatVec(&u->view, world, view);
	srpslMatVec(&u->projection, view, out->clipPosition);
	for (uint32_t k = 0; k < 3; ++k) srpslStoreF(out->varyings, k, world[k]);
	for (uint32_t k = 0; k < 3; ++k) srpslStoreF(out->varyings, 3 + k, wn[k]);
	srpslStoreU(out->varyings, 6, srpslLoadU(vtx, u->uvOffset));
	srpslStoreU(out->varyings, 7, srpslLoadU(vtx, u->uvOffset + 1));
	for (uint32_t w = 0; w < SRP_STD_MAX_PASS; ++w)
		if (w < u->extraCount)
			srpslStoreU(out->varyings, 8 + w, srpslLoadU(vtx, u->extraOffset + w));
}

/* Clip position as srpVsTransform; the varyings are `passCount` raw bytes of
 * the vertex starting at byte `passOffset` (both clamped to 64), so that a
 * program can hand any packed varying block (sub-word integers, doubles,
 * unaligned members) straight from its vertex layout to the interpolator. */
SRP_SHADER_FN void srpslVsBytes(SRPVertexShaderIn* in, SRPVertexShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	const unsigned char* vtx = (const unsigned char*) in->vertex;
	float p[4] = { srpslLoadF(vtx, 0), srpslLoadF(vtx, 1), srpslLoadF(vtx, 2), 1.0f };
	float a[4], b[4];
	srpslMatVec(&u->model, p, a);
	srpslMatVec(&u->view, a, b);
	srpslMatVec(&u->projection, b, out->clipPosition);
	const uint32_t off = u->passOffset < 64u ? u->passOffset : 64u;
	const uint32_t n = u->passCount < 64u ? u->passCount : 64u;
	memcpy((unsigned char*) out->varyings, vtx + off, n);
}

/* -------------------------------------------------------------- fragment */

SRP_SHADER_FN void srpslFsMixed(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	const unsigned char* v = (const unsigned char*) in->varyings + 4u * u->varyingOffset;
	int8_t a; double d[2]; uint16_t b; float f[2]; int16_t c; uint64_t e;
	memcpy(&a, v, 1); memcpy(d, v + 1, 16); memcpy(&b, v + 17, 2);
	memcpy(f, v + 19, 8); memcpy(&c, v + 27, 2); memcpy(&e, v + 29, 8);
	const uint32_t k = ((uint32_t) (int32_t) a * 7u + (uint32_t) b * 13u + (uint32_t) (int32_t) c * 3u + (uint32_t) e) & 15u;
	out->color[0] = (float) (d[0] - floor(d[0]));
	out->color[1] = 0.25f + 0.5f * (f[0] - floorf(f[0]));
	out->color[2] = 0.5f * (float) (d[1] - floor(d[1])) + 0.25f * (f[1] - floorf(f[1])) + (float) k * (0.25f / 15.0f);
	out->color[3] = 1.0f;
}

/* Colour of a uint8 varying at byte 4*varyingOffset: 0 red, 1 green, 2 blue
 * (the palette of the reference's flat-interpolation test scene), other
 * values hashed. */
SRP_SHADER_FN void srpslFsBytePalette(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	uint8_t k;
	memcpy(&k, (const unsigned char*) in->varyings + 4u * u->varyingOffset, 1);
	if (k < 3u) {
		for (int i = 0; i < 3; ++i) out->color[i] = (uint32_t) i == k ? 1.0f : 0.0f;
	} else {
		out->color[0] = (float) ((k * 37u) & 255u) / 255.0f;
		out->color[1] = (float) ((k * 101u) & 255u) / 255.0f;
		out->color[2] = (float) ((k * 193u) & 255u) / 255.0f;
	}
	out->color[3] = 1.0f;
}

/* ((id*97, id*57, id*23) mod 255) / 255 / colour[0] in double, then rounded to
 * float: the primitive-ID colouring of the reference's clipping, polygon-mode
 * and primitive test scenes (colour[0] = 1, or 2 for the darker variant). */
SRP_SHADER_FN void srpslFsPrimitiveMod(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	const uint32_t id = (uint32_t) in->primitiveID;
	const double div = (double) u->color[0];
	out->color[0] = (float) ((double) ((id * 97u) % 255u) / 255. / div);
	out->color[1] = (float) ((double) ((id * 57u) % 255u) / 255. / div);
	out->color[2] = (float) ((double) ((id * 23u) % 255u) / 255. / div);
	out->color[3] = 1.0f;
}

SRP_SHADER_FN void srpslFsVaryingColor(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	uint32_t o = u->varyingOffset;
	out->color[0] = srpslLoadF(in->varyings, o);
	out->color[1] = srpslLoadF(in->varyings, o + 1);
	out->color[2] = srpslLoadF(in->varyings, o + 2);
	out->color[3] = 1.0f;
}

SRP_SHADER_FN void srpslFsSolid(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	for (int k = 0; k < 4; ++k) out->color[k] = u->color[k];
}

/* Integer hash of the primitive ID, so that primitive numbering (which the
 * reference pins after clipping and culling) is visible in the image. */
SRP_SHADER_FN void srpslFsPrimitiveId(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	uint32_t id = (uint32_t) in->primitiveID;
	uint32_t r = (id * 37u + 11u) % 256u;
	uint32_t g = (id * 101u + 53u) % 256u;
	uint32_t b = (id * 193u + 97u) % 256u;
	out->color[0] = (float) r / 255.0f;
	out->color[1] = (float) g / 255.0f;
	out->color[2] = (float) b / 255.0f;
	out->color[3] = 1.0f;
}

SRP_SHADER_FN void srpslFsTexture(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	uint32_t o = u->varyingOffset;
	SRP_TEXTURE_SAMPLE(u->texture, srpslLoadF(in->varyings, o), srpslLoadF(in->varyings, o + 1), out->color);
}

/* Texture at a level of detail that grows with the distance: the texture
 * shrinks on screen as 1 / w (w = fragCoord[3], the interpolated clip w), so
 * lod = log2(max(1, texelScale * w)), texelScale being the texels a pixel
 * spans at w = 1. */
SRP_SHADER_FN void srpslFsTextureLod(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	uint32_t o = u->varyingOffset;
	float k = u->texelScale * in->fragCoord[3];
	float lod = k > 1.0f ? log2f(k) : 0.0f;
	SRP_TEXTURE_SAMPLE_LOD(u->texture, srpslLoadF(in->varyings, o), srpslLoadF(in->varyings, o + 1), lod, out->color);
}

SRP_SHADER_FN void srpslFsTextureModulate(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	uint32_t o = u->varyingOffset;
	float t[4];
	SRP_TEXTURE_SAMPLE(u->texture, srpslLoadF(in->varyings, o), srpslLoadF(in->varyings, o + 1), t);
	uint32_t id = srpslLoadU(in->varyings, o + 5);
	float tint = 0.6f + 0.4f * (float) ((id * 2654435761u) >> 24) / 255.0f;
	for (int k = 0; k < 3; ++k)
		out->color[k] = t[k] * srpslLoadF(in->varyings, o + 2 + k) * tint;
	out->color[3] = 1.0f;
}

/* Textured Blinn-Phong with the uniform's lights; varyings from srpVsWorld. */
SRP_SHADER_FN void srpslFsBlinnPhong(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	float pos[3], n[3], albedo[4];
	for (uint32_t k = 0; k < 3; ++k) { pos[k] = srpslLoadF(in->varyings, k); n[k] = srpslLoadF(in->varyings, 3 + k); }
	srpslNormalize3(n);
	if (u->texture)
		SRP_TEXTURE_SAMPLE(u->texture, srpslLoadF(in->varyings, 6), srpslLoadF(in->varyings, 7), albedo);
	else
		for (int k = 0; k < 4; ++k) albedo[k] = u->color[k];
	float v[3] = { u->cameraPos[0] - pos[0], u->cameraPos[1] - pos[1], u->cameraPos[2] - pos[2] };
	srpslNormalize3(v);
	float rgb[3] = { albedo[0] * u->ambient[0], albedo[1] * u->ambient[1], albedo[2] * u->ambient[2] };
	uint32_t nl = u->nLights < SRP_STD_MAX_LIGHTS ? u->nLights : SRP_STD_MAX_LIGHTS;
	for (uint32_t i = 0; i < nl; ++i)
	{
		float l[3] = { u->lightPos[i][0] - pos[0], u->lightPos[i][1] - pos[1], u->lightPos[i][2] - pos[2] };
		srpslNormalize3(l);
		float h[3] = { l[0] + v[0], l[1] + v[1], l[2] + v[2] };
		srpslNormalize3(h);
		float nd = srpslDot3(n, l);
		float diff = nd > 0.0f ? nd : 0.0f;
		float nh = srpslDot3(n, h);
		float spec = (nd > 0.0f && nh > 0.0f) ? powf(nh, u->shininess) : 0.0f;
		for (int k = 0; k < 3; ++k)
			rgb[k] += (albedo[k] * diff + spec) * u->lightColor[i][k];
	}
	for (int k = 0; k < 3; ++k) out->color[k] = srpslClamp01(rgb[k]);
	out->color[3] = 1.0f;
}

/* Lattice hash for value noise (integer only, identical on host and device). */
SRP_SHADER_FN float srpslLattice(int32_t x, int32_t y, int32_t z)
{
	uint32_t h = (uint32_t) x * 73856093u ^ (uint32_t) y * 19349663u ^ (uint32_t) z * 83492791u;
	h ^= h >> 13; h *= 0x5bd1e995u; h ^= h >> 15;
	return (float) (h & 0xFFFFFFu) * (1.0f / 16777215.0f);
}

SRP_SHADER_FN float srpslSmooth(float t) { return t * t * (3.0f - 2.0f * t); }

SRP_SHADER_FN float srpslValueNoise(float x, float y, float z)
{
	float fx = floorf(x), fy = floorf(y), fz = floorf(z);
	int32_t ix = (int32_t) fx, iy = (int32_t) fy, iz = (int32_t) fz;
	float tx = srpslSmooth(x - fx), ty = srpslSmooth(y - fy), tz = srpslSmooth(z - fz);
	float c[2][2][2];
	for (int a = 0; a < 2; ++a) for (int b = 0; b < 2; ++b) for (int d = 0; d < 2; ++d)
		c[a][b][d] = srpslLattice(ix + a, iy + b, iz + d);
	float x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * tx;
	float x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * tx;
	float x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * tx;
	float x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * tx;
	float y0 = x00 + (x10 - x00) * ty;
	float y1 = x01 + (x11 - x01) * ty;
	return y0 + (y1 - y0) * tz;
}

/* The expensive procedural shader: fractal value-noise marble albedo lit by
 * up to 16 point lights (Blinn-Phong). Varyings from srpVsWorld. */
SRP_SHADER_FN void srpslFsMarble(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	float pos[3], n[3];
	for (uint32_t k = 0; k < 3; ++k) { pos[k] = srpslLoadF(in->varyings, k); n[k] = srpslLoadF(in->varyings, 3 + k); }
	srpslNormalize3(n);
	float f = u->marbleFrequency, amp = 1.0f, turb = 0.0f, norm = 0.0f;
	uint32_t oct = u->marbleOctaves < 12u ? u->marbleOctaves : 12u;
	for (uint32_t i = 0; i < oct; ++i)
	{
		turb += amp * srpslValueNoise(pos[0] * f, pos[1] * f, pos[2] * f);
		norm += amp;
		f *= 2.0f;
		amp *= u->marbleGain;
	}
	turb = norm > 0.0f ? turb / norm : 0.0f;
	float s = 0.5f + 0.5f * sinf((pos[0] + pos[1] * 0.5f) * u->marbleFrequency + 6.0f * turb);
	float vein = s * s * s;
	float albedo[3] = { 0.90f - 0.55f * vein, 0.88f - 0.60f * vein, 0.84f - 0.45f * vein };
	float v[3] = { u->cameraPos[0] - pos[0], u->cameraPos[1] - pos[1], u->cameraPos[2] - pos[2] };
	srpslNormalize3(v);
	float rgb[3] = { albedo[0] * u->ambient[0], albedo[1] * u->ambient[1], albedo[2] * u->ambient[2] };
	uint32_t nl = u->nLights < SRP_STD_MAX_LIGHTS ? u->nLights : SRP_STD_MAX_LIGHTS;
	for (uint32_t i = 0; i < nl; ++i)
	{
		float l[3] = { u->lightPos[i][0] - pos[0], u->lightPos[i][1] - pos[1], u->lightPos[i][2] - pos[2] };
		float d2 = srpslDot3(l, l);
		srpslNormalize3(l);
		float h[3] = { l[0] + v[0], l[1] + v[1], l[2] + v[2] };
		srpslNormalize3(h);
		float nd = srpslDot3(n, l);
		float diff = nd > 0.0f ? nd : 0.0f;
		float nh = srpslDot3(n, h);
		float spec = (nd > 0.0f && nh > 0.0f) ? powf(nh, u->shininess) : 0.0f;
		float att = 1.0f / (1.0f + 0.05f * d2);
		for (int k = 0; k < 3; ++k)
			rgb[k] += (albedo[k] * diff + 0.5f * spec) * u->lightColor[i][k] * att;
	}
	for (int k = 0; k < 3; ++k) out->color[k] = srpslClamp01(rgb[k]);
	out->color[3] = 1.0f;
}

/* Late-Z shader: colour from varyings, fragDepth = depth * scale + bias. */
SRP_SHADER_FN void srpslFsDepthOverwrite(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	srpslFsVaryingColor(in, out);
	out->fragDepth = in->fragCoord[2] * u->depthScale + u->depthBias;
}

SRP_SHADER_FN void srpslFsFragCoord(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	out->color[0] = in->fragCoord[0] * (1.0f / 1024.0f);
	out->color[1] = in->fragCoord[1] * (1.0f / 1024.0f);
	float z = in->fragCoord[2] * 4.0f;
	out->color[2] = z - floorf(z);
	out->color[3] = in->frontFacing ? 1.0f : 0.5f;
}

SRP_SHADER_FN void srpslFsFlatInt(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	const SRPStdUniform* u = (const SRPStdUniform*) in->uniform;
	int32_t v = (int32_t) srpslLoadU(in->varyings, u->varyingOffset);
	uint32_t k = (uint32_t) v;
	out->color[0] = (float) ((k * 53u) % 7u) / 6.0f;
	out->color[1] = (float) ((k * 29u) % 5u) / 4.0f;
	out->color[2] = (float) ((k * 17u) % 3u) / 2.0f;
	out->color[3] = 1.0f;
}
