/* srp-gb300 public API umbrella header (replaces include/srp/srp.h of
 * kitrofimov/srp, srp.h:9-21). Define SRP_INCLUDE_VEC / SRP_INCLUDE_MAT before
 * including it to also get the math types and helpers. */
#pragma once

#include "srp/context.h"
#include "srp/buffer.h"
#include "srp/texture.h"
#include "srp/color.h"
#include "srp/framebuffer.h"
#include "srp/vertex.h"
#include "srp/shaders.h"

#ifdef SRP_INCLUDE_VEC
#include "srp/vec.h"
#endif
#ifdef SRP_INCLUDE_MAT
#include "srp/mat.h"
#endif
