/* srp-gb300 public API: opaque vertex / varying types and varying metadata.
 *
 * Replaces include/srp/vertex.h of kitrofimov/srp (vertex.h:24-46). */
#pragma once

#include <stddef.h>
#include "srp/type.h"

/** User vertex record as stored in a vertex buffer (opaque to the library). */
typedef struct SRPVertex SRPVertex;

/** Per-vertex shader outputs (opaque byte block of varyingsSize bytes). */
typedef struct SRPVarying SRPVarying;

/** How a varying is interpolated across a primitive. */
typedef enum SRPInterpolationMode
{
	SRP_INTERPOLATION_MODE_PERSPECTIVE,
	SRP_INTERPOLATION_MODE_AFFINE,
	SRP_INTERPOLATION_MODE_FLAT
} SRPInterpolationMode;

/** Layout of one varying: nItems elements of `type`, packed back to back with
 *  the other varyings in declaration order (no padding). */
typedef struct
{
	size_t nItems;
	SRPType type;
	SRPInterpolationMode interpolationMode;
} SRPVaryingInfo;

/** Interpolated varyings as seen by the fragment shader (same byte layout as
 *  SRPVarying). */
typedef struct SRPInterpolated SRPInterpolated;
