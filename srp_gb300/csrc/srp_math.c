/* Host vec/mat helpers of the public API (srp/vec.h, srp/mat.h).
 *
 * The arithmetic restates kitrofimov/srp src/math/vec.c:16-189 and
 * src/math/mat.c:16-215 step for step: every sum is evaluated left to right in
 * fp32 without contraction (build with -ffp-contract=off), and the angle-based
 * constructors evaluate sin/cos products in double before narrowing to float,
 * because scene matrices built here feed vertex positions and so coverage.
 * Compiled into both the GPU library and the CPU oracle. */
#include <math.h>
#include "srp/vec.h"
#include "srp/mat.h"

static vec2 mk2(float x, float y) { vec2 r; r.x = x; r.y = y; return r; }
static vec3 mk3(float x, float y, float z) { vec3 r; r.x = x; r.y = y; r.z = z; return r; }
static vec4 mk4(float x, float y, float z, float w) { vec4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }

vec2 vec2Add(vec2 a, vec2 b) { return mk2(a.x + b.x, a.y + b.y); }
vec2 vec2Subtract(vec2 a, vec2 b) { return mk2(a.x - b.x, a.y - b.y); }
float vec2DotProduct(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
vec2 vec2MultiplyScalar(vec2 a, float b) { return mk2(a.x * b, a.y * b); }
vec2 vec2Negate(vec2 v) { return mk2(-v.x, -v.y); }
vec2 vec2MultiplyVec2(vec2 a, vec2 b) { return mk2(a.x * b.x, a.y * b.y); }
vec2 vec2Normalize(vec2 v)
{
	float len = sqrtf(v.x * v.x + v.y * v.y);
	if (!(len > 0)) return mk2(0, 0);
	float inv = 1.0f / len;
	return mk2(v.x * inv, v.y * inv);
}
vec2 vec2Reflect(vec2 i, vec2 n)
{
	float d = vec2DotProduct(n, i);
	return vec2Subtract(i, vec2MultiplyScalar(n, 2.f * d));
}

vec3 vec3Add(vec3 a, vec3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
vec3 vec3Subtract(vec3 a, vec3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
float vec3DotProduct(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
vec3 vec3MultiplyScalar(vec3 a, float b) { return mk3(a.x * b, a.y * b, a.z * b); }
vec3 vec3Negate(vec3 v) { return mk3(-v.x, -v.y, -v.z); }
vec3 vec3MultiplyVec3(vec3 a, vec3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
vec3 vec3Normalize(vec3 v)
{
	float len = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
	if (!(len > 0)) return mk3(0, 0, 0);
	float inv = 1 / len;
	return mk3(v.x * inv, v.y * inv, v.z * inv);
}
vec3 vec3Reflect(vec3 i, vec3 n)
{
	float d = vec3DotProduct(n, i);
	return vec3Subtract(i, vec3MultiplyScalar(n, 2.f * d));
}

vec4 vec4Add(vec4 a, vec4 b) { return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
vec4 vec4Subtract(vec4 a, vec4 b) { return mk4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
float vec4DotProduct(vec4 a, vec4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
vec4 vec4MultiplyScalar(vec4 a, float b) { return mk4(a.x * b, a.y * b, a.z * b, a.w * b); }
vec4 vec4Negate(vec4 v) { return mk4(-v.x, -v.y, -v.z, -v.w); }
vec4 vec4MultiplyVec4(vec4 a, vec4 b) { return mk4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
vec4 vec4Normalize(vec4 v)
{
	float len = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w);
	if (!(len > 0)) return mk4(0, 0, 0, 0);
	float inv = 1.0f / len;
	return mk4(v.x * inv, v.y * inv, v.z * inv, v.w * inv);
}
vec4 vec4Reflect(vec4 i, vec4 n)
{
	float d = vec4DotProduct(n, i);
	return vec4Subtract(i, vec4MultiplyScalar(n, 2.f * d));
}

vec4 mat4MultiplyVec4(const mat4* SRP_RESTRICT m, vec4 v)
{
	vec4 r;
	for (int i = 0; i < 4; ++i)
		r.v[i] = m->data[i][0] * v.x + m->data[i][1] * v.y + m->data[i][2] * v.z + m->data[i][3] * v.w;
	return r;
}

mat4 mat4MultiplyMat4(const mat4* SRP_RESTRICT a, const mat4* SRP_RESTRICT b)
{
	mat4 r;
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j)
			r.data[i][j] = a->data[i][0] * b->data[0][j] + a->data[i][1] * b->data[1][j]
			             + a->data[i][2] * b->data[2][j] + a->data[i][3] * b->data[3][j];
	return r;
}

static mat4 diag(float a, float b, float c, float d)
{
	mat4 r = {{{0}}};
	r.data[0][0] = a; r.data[1][1] = b; r.data[2][2] = c; r.data[3][3] = d;
	return r;
}

mat4 mat4ConstructIdentity(void) { return diag(1, 1, 1, 1); }
mat4 mat4ConstructScale(float x, float y, float z) { return diag(x, y, z, 1); }

mat4 mat4ConstructTranslate(float x, float y, float z)
{
	mat4 r = diag(1, 1, 1, 1);
	r.data[0][3] = x; r.data[1][3] = y; r.data[2][3] = z;
	return r;
}

/* Rotation X then Y then Z folded into one matrix; each entry is a product of
 * double sines/cosines evaluated left to right, then narrowed to float. */
mat4 mat4ConstructRotate(float x, float y, float z)
{
	const double sx = sin(x), cx = cos(x), sy = sin(y), cy = cos(y), sz = sin(z), cz = cos(z);
	mat4 r = {{{0}}};
	r.data[0][0] = cy * cz;
	r.data[0][1] = sx * sy * cz - cx * sz;
	r.data[0][2] = cx * sy * cz + sx * sz;
	r.data[1][0] = cy * sz;
	r.data[1][1] = sx * sy * sz + cx * cz;
	r.data[1][2] = cx * sy * sz - sx * cz;
	r.data[2][0] = -sy;
	r.data[2][1] = sx * cy;
	r.data[2][2] = cx * cy;
	r.data[3][3] = 1;
	return r;
}

mat4 mat4ConstructTRS(float tx, float ty, float tz, float rx, float ry, float rz,
                      float sx, float sy, float sz)
{
	mat4 t = mat4ConstructTranslate(tx, ty, tz);
	mat4 rot = mat4ConstructRotate(rx, ry, rz);
	mat4 s = mat4ConstructScale(sx, sy, sz);
	mat4 rs = mat4MultiplyMat4(&rot, &s);
	return mat4MultiplyMat4(&t, &rs);
}

mat4 mat4ConstructView(float cx, float cy, float cz, float rx, float ry, float rz,
                       float sx, float sy, float sz)
{
	return mat4ConstructTRS(-cx, -cy, -cz, -rx, -ry, -rz, sx, sy, sz);
}

mat4 mat4ConstructOrthogonalProjection(float x0, float x1, float y0, float y1, float z0, float z1)
{
	mat4 r = {{{0}}};
	r.data[0][0] = 2 / (x1 - x0);
	r.data[0][3] = -(x1 + x0) / (x1 - x0);
	r.data[1][1] = 2 / (y1 - y0);
	r.data[1][3] = -(y1 + y0) / (y1 - y0);
	r.data[2][2] = 2 / (z1 - z0);
	r.data[2][3] = -(z1 + z0) / (z1 - z0);
	r.data[3][3] = 1;
	return r;
}

/* Frustum-to-box map (near, far) followed by the orthographic box-to-cube
 * map, multiplied as ortho * persp like the reference. */
mat4 mat4ConstructPerspectiveProjection(float x0, float x1, float y0, float y1, float zn, float zf)
{
	mat4 p = {{{0}}};
	p.data[0][0] = zn;
	p.data[1][1] = zn;
	p.data[2][2] = zn + zf;
	p.data[2][3] = -zn * zf;
	p.data[3][2] = 1;
	mat4 o = mat4ConstructOrthogonalProjection(x0, x1, y0, y1, zn, zf);
	return mat4MultiplyMat4(&o, &p);
}
