/* srp-gb300 public API: packed float vectors.
 *
 * Replaces include/srp/vec.h of kitrofimov/srp (vec.h:15-104). The unions are
 * byte-packed (alignment 1) exactly as in the reference, so user vertex
 * structs keep the same size and offsets. */
#pragma once

#include <stdint.h>

#pragma pack(push, 1)

typedef union vec2 {
	struct { float x, y; };
	float v[2];
} vec2;

typedef union vec3 {
	struct { float x, y, z; };
	struct { vec2 xy; float _z; };
	struct { float _x; vec2 yz; };
	float v[3];
} vec3;

typedef union vec4 {
	struct { float x, y, z, w; };
	struct { vec2 xy; float _z, _w; };
	struct { float _x; vec2 yz; float __w; };
	struct { float __x, _y; vec2 zw; };
	struct { vec3 xyz; float ___w; };
	struct { float ___x; vec3 yzw; };
	float v[4];
} vec4;

/* Compound-literal constructors and swizzles (C only). */
#define VEC2(x, y)           ((vec2) {{x, y}})
#define VEC3(x, y, z)        ((vec3) {{x, y, z}})
#define VEC4(x, y, z, w)     ((vec4) {{x, y, z, w}})
#define VEC4_FROM_VEC3(v, a) ((vec4) {.xyz = (v), .___w = (a)})
#define SWZ2(v, a, b)       ((vec2) {{(v).a, (v).b}})
#define SWZ3(v, a, b, c)    ((vec3) {{(v).a, (v).b, (v).c}})
#define SWZ4(v, a, b, c, d) ((vec4) {{(v).a, (v).b, (v).c, (v).d}})

#pragma pack(pop)

#ifdef __cplusplus
extern "C" {
#endif

/* Component-wise helpers (vec.h:56-104): plain fp32 arithmetic, no FMA. */
vec2 vec2Add(vec2 a, vec2 b);
vec2 vec2Subtract(vec2 a, vec2 b);
float vec2DotProduct(vec2 a, vec2 b);
vec2 vec2MultiplyScalar(vec2 a, float b);
vec2 vec2Normalize(vec2 v);
vec2 vec2Reflect(vec2 i, vec2 n);
vec2 vec2MultiplyVec2(vec2 a, vec2 b);
vec2 vec2Negate(vec2 v);

vec3 vec3Add(vec3 a, vec3 b);
vec3 vec3Subtract(vec3 a, vec3 b);
float vec3DotProduct(vec3 a, vec3 b);
vec3 vec3MultiplyScalar(vec3 a, float b);
vec3 vec3Normalize(vec3 v);
vec3 vec3Reflect(vec3 i, vec3 n);
vec3 vec3MultiplyVec3(vec3 a, vec3 b);
vec3 vec3Negate(vec3 v);

vec4 vec4Add(vec4 a, vec4 b);
vec4 vec4Subtract(vec4 a, vec4 b);
float vec4DotProduct(vec4 a, vec4 b);
vec4 vec4MultiplyScalar(vec4 a, float b);
vec4 vec4Normalize(vec4 v);
vec4 vec4Reflect(vec4 i, vec4 n);
vec4 vec4MultiplyVec4(vec4 a, vec4 b);
vec4 vec4Negate(vec4 v);

#ifdef __cplusplus
}
#endif
