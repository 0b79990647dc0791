/* srp-gb300 public API: opaque scratch-allocator handle kept in SRPContext.
 *
 * Replaces include/srp/arena.h of kitrofimov/srp (arena.h:13-14). The GPU build
 * replaces the per-draw host arena with device-resident pools owned by the
 * library; the pointer stays in SRPContext only to keep the struct layout. */
#pragma once

typedef struct SRPArena SRPArena;
