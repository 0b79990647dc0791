/* srp-gb300 public API: 8-bit RGBA colour.
 *
 * Replaces include/srp/color.h of kitrofimov/srp (color.h:15-19). Colour
 * buffer words are packed R<<24 | G<<16 | B<<8 | A. */
#pragma once

#include <stdint.h>

typedef struct SRPColor
{
	uint8_t r, g, b, a;
} SRPColor;
