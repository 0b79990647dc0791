/* srp-gb300 public API: textures (nearest sampling as the reference; bilinear
 * and trilinear filtering as additions).
 *
 * Replaces include/srp/texture.h of kitrofimov/srp (texture.h:18-67). Texels
 * are stored as 3 channels (RGB8) like the reference; the alpha read back by
 * srpTextureGetFilteredColor is always 1. srpNewTexture reads binary PPM (P6)
 * and PNG (8-bit RGB/RGBA, non-interlaced); srpNewTextureFromMemory is an
 * addition of this library. */
#pragma once

#include <stdint.h>
#include <stddef.h>
#include "srp/color.h"

typedef enum
{
	TW_REPEAT,
	TW_CLAMP_TO_EDGE
} SRPTextureWrappingMode;

typedef struct SRPTexture SRPTexture;

typedef enum SRPTextureParameter
{
	SRP_TEXTURE_WRAPPING_MODE_X,
	SRP_TEXTURE_WRAPPING_MODE_Y
} SRPTextureParameter;

#ifdef __cplusplus
extern "C" {
#endif

SRPTexture* srpNewTexture(const char* image, SRPTextureWrappingMode wrappingModeX,
                          SRPTextureWrappingMode wrappingModeY);              /* texture.h:32-36 */
void srpFreeTexture(SRPTexture* tex);                                         /* texture.h:39 */
/** Host-side lookup with the texture's filter (the reference's nearest texel
 *  by default); out = RGBA in [0, 1] (texture.h:46-48). The same arithmetic
 *  runs on the device inside fragment shaders. */
void srpTextureGetFilteredColor(const SRPTexture* tex, float u, float v, float out[4]);
int srpTextureGet(SRPTexture* tex, SRPTextureParameter parameter);            /* texture.h:62 */
void srpTextureSet(SRPTexture* tex, SRPTextureParameter parameter, int data); /* texture.h:67 */

/** Addition: texture filtering. The reference samples the nearest texel
 *  only; bilinear filtering and mipmapping are items of its to-do list
 *  (README.md:71-72). With u, v wrapped as for the nearest texel and
 *  x = (w - 1) * u, y = (h - 1) * (1 - v) on a level of w x h texels:
 *  - NEAREST (the default) is the reference's sampling, unchanged;
 *  - BILINEAR blends the texels (floor(x), floor(y)) and (+1, +1) with the
 *    fractions of x and y (the +1 neighbour wraps or clamps like u and v);
 *  - TRILINEAR samples a mip chain bilinearly at two levels and blends them:
 *    level l + 1 is the 2x2 box average of level l, (a + b + c + d + 2) / 4
 *    per channel, w and h halved and rounded down (at least 1); the level
 *    of detail comes from srpTextureGetFilteredColorLod, clamped to the
 *    chain, and srpTextureGetFilteredColor samples level 0. */
typedef enum SRPTextureFilter
{
	SRP_TEXTURE_FILTER_NEAREST,
	SRP_TEXTURE_FILTER_BILINEAR,
	SRP_TEXTURE_FILTER_TRILINEAR
} SRPTextureFilter;

void srpTextureSetFilter(SRPTexture* tex, SRPTextureFilter filter);
SRPTextureFilter srpTextureGetFilter(const SRPTexture* tex);
/** srpTextureGetFilteredColor at level of detail lod (used by TRILINEAR). */
void srpTextureGetFilteredColorLod(const SRPTexture* tex, float u, float v, float lod, float out[4]);
/** Levels of the mip chain of a w x h texture (1 + floor(log2(max(w, h)))). */
int srpTextureMipLevels(int width, int height);

/** Addition: build a texture from `channels`-per-texel 8-bit data (channels
 *  3 or 4, row-major, top row first); only RGB is kept, as the reference
 *  keeps 3 channels. Returns NULL (and reports) on bad arguments. */
SRPTexture* srpNewTextureFromMemory(const uint8_t* texels, int width, int height, int channels,
                                    SRPTextureWrappingMode wrappingModeX,
                                    SRPTextureWrappingMode wrappingModeY);

#ifdef __cplusplus
}
#endif
