/* srp-gb300 public API: textures (nearest sampling).
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
/** Host-side nearest lookup; out = RGBA in [0, 1] (texture.h:46-48). The same
 *  arithmetic runs on the device inside fragment shaders. */
void srpTextureGetFilteredColor(const SRPTexture* tex, float u, float v, float out[4]);
int srpTextureGet(SRPTexture* tex, SRPTextureParameter parameter);            /* texture.h:62 */
void srpTextureSet(SRPTexture* tex, SRPTextureParameter parameter, int data); /* texture.h:67 */

/** Addition: build a texture from `channels`-per-texel 8-bit data (channels
 *  3 or 4, row-major, top row first); only RGB is kept, as the reference
 *  keeps 3 channels. Returns NULL (and reports) on bad arguments. */
SRPTexture* srpNewTextureFromMemory(const uint8_t* texels, int width, int height, int channels,
                                    SRPTextureWrappingMode wrappingModeX,
                                    SRPTextureWrappingMode wrappingModeY);

#ifdef __cplusplus
}
#endif
