/* Device helpers that reproduce the reference's per-fragment arithmetic.
 *
 * Everything that can change coverage, depth or stencil is written with the
 * same operations, operand order and precision as kitrofimov/srp (cited per
 * function); the translation units that include this header are compiled with
 * -fmad=false so no multiply-add is ever fused. */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "gpu_types.h"
#include "chain.h"
#include "srp/shaders.h"
#include "srp/context.h"
#include "srp/type.h"

namespace srpg {

/* ROUGHLY_ZERO(x) = fabs((double) x) <= 1e-9 (src/math/utils.h:41-45). For a
 * float x this is |x| <= 1e-9f, 1e-9f being the largest float not above 1e-9. */
__device__ __forceinline__ bool roughlyZero(float x) { return fabsf(x) <= 1e-9f; }

/* NDC -> screen space in double, then narrowed (src/core/framebuffer.c:48-55). */
__device__ __forceinline__ void ndcToScreen(int W, int H, float nx, float ny, float& sx, float& sy)
{
	sx = (float) (((double) (float) W / 2.) * ((double) nx + 1.));
	sy = (float) (((double) (float) H / 2.) * (1. - (double) ny));
}

/* invW = (float)(1.0 / (double) w): a float quotient computed in double and
 * rounded once more to float equals the correctly rounded float quotient
 * (53 >= 2*24 + 2), so the IEEE reciprocal is used. */
__device__ __forceinline__ float invW(float w) { return __frcp_rn(w); }

__device__ __forceinline__ bool stencilCompare(uint32_t ref, uint32_t stored, uint32_t mask, int op)
{
	/* src/raster/fragment.c:156-178 */
	const uint32_t l = ref & mask & 0xFFu, r = stored & mask & 0xFFu;
	switch (op) {
	case SRP_COMPARE_NEVER: return false;
	case SRP_COMPARE_ALWAYS: return true;
	case SRP_COMPARE_LESS: return l < r;
	case SRP_COMPARE_LEQUAL: return l <= r;
	case SRP_COMPARE_GREATER: return l > r;
	case SRP_COMPARE_GEQUAL: return l >= r;
	case SRP_COMPARE_EQUAL: return l == r;
	case SRP_COMPARE_NOTEQUAL: return l != r;
	default: return false;
	}
}

__device__ __forceinline__ uint32_t stencilApply(int op, uint32_t s, uint32_t ref, uint32_t writeMask)
{
	/* src/raster/fragment.c:180-223: new value through the write mask */
	uint32_t v;
	switch (op) {
	case SRP_STENCIL_KEEP: v = s; break;
	case SRP_STENCIL_ZERO: v = 0; break;
	case SRP_STENCIL_REPLACE: v = ref; break;
	case SRP_STENCIL_INCR: v = s < 255u ? s + 1u : 255u; break;
	case SRP_STENCIL_INCR_WRAP: v = (s + 1u) & 0xFFu; break;
	case SRP_STENCIL_DECR: v = s > 0u ? s - 1u : 0u; break;
	case SRP_STENCIL_DECR_WRAP: v = (s - 1u) & 0xFFu; break;
	case SRP_STENCIL_INVERT: v = (~s) & 0xFFu; break;
	default: v = s; break;
	}
	return ((s & ~writeMask) | (v & writeMask)) & 0xFFu;
}

__device__ __forceinline__ bool depthCompare(int op, float in, float stored)
{
	/* src/raster/fragment.c:225-245 (caller handles the disabled test) */
	switch (op) {
	case SRP_COMPARE_NEVER: return false;
	case SRP_COMPARE_ALWAYS: return true;
	case SRP_COMPARE_LESS: return in < stored;
	case SRP_COMPARE_LEQUAL: return in <= stored;
	case SRP_COMPARE_GREATER: return in > stored;
	case SRP_COMPARE_GEQUAL: return in >= stored;
	case SRP_COMPARE_EQUAL: return in == stored;
	case SRP_COMPARE_NOTEQUAL: return in != stored;
	default: return false;
	}
}

/* Scissor test on logical pixel coordinates with size_t semantics
 * (src/raster/fragment.c:127-140). */
__device__ __forceinline__ bool scissorPass(const DrawState& st, int x, int y)
{
	if (!st.scissorEnabled) return true;
	const uint64_t ux = (uint64_t) (int64_t) x, uy = (uint64_t) (int64_t) y;
	return !(ux < st.sx0 || ux >= st.sx1 || uy < st.sy0 || uy >= st.sy1);
}

/* clamp(c * 255) truncated to 8 bits, packed R<<24|G<<16|B<<8|A
 * (src/core/color.c:14-23). */
__device__ __forceinline__ uint32_t packColor(const float c[4])
{
	uint32_t r = 0;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		const float v = __fmul_rn(c[k], 255.0f);
		const float cl = (v < 0.0f) ? 0.0f : (v > 255.0f) ? 255.0f : v;
		r = (r << 8) | ((uint32_t) cl & 0xFFu);
	}
	return r;
}

/* Bilinear sample of mip level l at wrapped (u, v): x = (w - 1) u,
 * y = (h - 1)(1 - v), the texels at floor(x), floor(y) and +1 (the +1
 * neighbour wraps or clamps) blended by the fractions, per channel in
 * 0..255 (srpTextureSetFilter's definition, srp/texture.h). */
__device__ __forceinline__ void textureBilinear(const TextureDesc* t, int l, float u, float v, float c[3])
{
	const int w = t->lw[l], h = t->lh[l];
	const float x = __fmul_rn((float) (w - 1), u), y = __fmul_rn((float) (h - 1), __fsub_rn(1.0f, v));
	const float fx0 = floorf(x), fy0 = floorf(y);
	int x0 = (int) fx0, y0 = (int) fy0;
	x0 = min(max(x0, 0), w - 1);
	y0 = min(max(y0, 0), h - 1);
	const float fx = __fsub_rn(x, fx0), fy = __fsub_rn(y, fy0);
	const int x1 = x0 + 1 < w ? x0 + 1 : (t->wrapX == 0 ? 0 : w - 1);
	const int y1 = y0 + 1 < h ? y0 + 1 : (t->wrapY == 0 ? 0 : h - 1);
	const uint32_t* L = t->texels + t->loff[l];
	const uint32_t a = __ldg(L + (size_t) y0 * w + x0), b = __ldg(L + (size_t) y0 * w + x1);
	const uint32_t d = __ldg(L + (size_t) y1 * w + x0), e = __ldg(L + (size_t) y1 * w + x1);
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		const float ta = (float) ((a >> (8 * k)) & 0xFFu), tb = (float) ((b >> (8 * k)) & 0xFFu);
		const float td = (float) ((d >> (8 * k)) & 0xFFu), te = (float) ((e >> (8 * k)) & 0xFFu);
		const float top = __fadd_rn(ta, __fmul_rn(fx, __fsub_rn(tb, ta)));
		const float bot = __fadd_rn(td, __fmul_rn(fx, __fsub_rn(te, td)));
		c[k] = __fadd_rn(top, __fmul_rn(fy, __fsub_rn(bot, top)));
	}
}

/* Filtered sample at level of detail lod: NEAREST and BILINEAR read level 0,
 * TRILINEAR blends the bilinear samples of floor(lod) and the next level
 * (lod clamped to the chain). */
__device__ __forceinline__ void textureFiltered(const TextureDesc* t, float u, float v, float lod, float out[4])
{
	if (u < 0.0f || u > 1.0f) u = t->wrapX == 0 ? __fsub_rn(u, floorf(u)) : fmaxf(0.0f, fminf(1.0f, u));
	if (v < 0.0f || v > 1.0f) v = t->wrapY == 0 ? __fsub_rn(v, floorf(v)) : fmaxf(0.0f, fminf(1.0f, v));
	float c[3];
	textureBilinear(t, 0, u, v, c);
	if (t->filter == 2 && t->nLevels > 1) {
		const float top = (float) (t->nLevels - 1);
		const float ld = lod > 0.0f ? (lod < top ? lod : top) : 0.0f;   /* NaN: level 0 */
		const int l0 = (int) floorf(ld);
		const float f = __fsub_rn(ld, (float) l0);
		float c0[3], c1[3];
		textureBilinear(t, l0, u, v, c0);
		textureBilinear(t, l0 + 1 < t->nLevels ? l0 + 1 : l0, u, v, c1);
#pragma unroll
		for (int k = 0; k < 3; ++k) c[k] = __fadd_rn(c0[k], __fmul_rn(f, __fsub_rn(c1[k], c0[k])));
	}
	const float inv255 = (float) (1. / 255.);
#pragma unroll
	for (int k = 0; k < 3; ++k) out[k] = __fmul_rn(c[k], inv255);
	out[3] = 1.0f;
}

/* Nearest texel with the reference's wrap rules (src/core/texture.c:56-81);
 * textures set to a filter go to textureFiltered at level 0. */
__device__ __forceinline__ void textureSample(const TextureDesc* t, float u, float v, float out[4])
{
	if (t->filter != 0) { textureFiltered(t, u, v, 0.0f, out); return; }
	if (u < 0.0f || u > 1.0f) u = t->wrapX == 0 ? __fsub_rn(u, floorf(u)) : fmaxf(0.0f, fminf(1.0f, u));
	if (v < 0.0f || v > 1.0f) v = t->wrapY == 0 ? __fsub_rn(v, floorf(v)) : fmaxf(0.0f, fminf(1.0f, v));
	const float x = __fmul_rn((float) t->wm1, u);
	const float y = __fmul_rn((float) t->hm1, __fsub_rn(1.0f, v));
	const unsigned long long xi = (unsigned long long) ((double) x + 0.5);
	const unsigned long long yi = (unsigned long long) ((double) y + 0.5);
	unsigned long long idx = xi + yi * (unsigned long long) t->width;
	const unsigned long long n = (unsigned long long) t->width * (unsigned long long) t->height;
	if (idx >= n) idx = n - 1;  /* NaN coordinates only; the reference reads out of bounds */
	const uint32_t texel = __ldg(t->texels + idx);
	const float inv255 = (float) (1. / 255.);
	out[0] = __fmul_rn((float) (texel & 0xFFu), inv255);
	out[1] = __fmul_rn((float) ((texel >> 8) & 0xFFu), inv255);
	out[2] = __fmul_rn((float) ((texel >> 16) & 0xFFu), inv255);
	out[3] = 1.0f;
}

/* srpTextureGetFilteredColorLod on the device. */
__device__ __forceinline__ void textureSampleLod(const TextureDesc* t, float u, float v, float lod, float out[4])
{
	if (t->filter == 0) textureSample(t, u, v, out);
	else textureFiltered(t, u, v, lod, out);
}

/* ------------------------------------------------------------ varyings */

__device__ __forceinline__ float ldf(const uint32_t* p) { return __uint_as_float(*p); }

/* Interpolate the varyings of a primitive with n vertices (3: triangle,
 * 2: line) into out[] (src/pipeline/interpolation.c:63-163). Every floating
 * element starts from 0 and accumulates vertex by vertex, as the reference
 * does; integer elements are copied from the provoking vertex. `affineOnly`
 * is the clipping case (invW == NULL in the reference). */
template <int N>
__device__ __forceinline__ void interpolateWords(const VaryingLayout& L, const uint32_t* vary, const uint32_t vref[N],
                                                 const float w[N], const float iw[N], float recip, bool provFirst,
                                                 bool affineOnly, uint32_t out[kMaxVaryingWords])
{
	const int prov = provFirst ? 0 : N - 1;
	const int nw = L.nWords;
#pragma unroll
	for (int k = 0; k < kMaxVaryingWords; ++k) {
		if (k < nw) {
			const int mode = L.wordMode[k];
			if (!L.wordIsFloat[k]) {
				out[k] = vary[(size_t) vref[prov] * nw + k];
			} else if (mode == kPerspective && !affineOnly) {
				float v = 0.0f;
#pragma unroll
				for (int i = 0; i < N; ++i)
					v = __fadd_rn(v, __fmul_rn(__fmul_rn(ldf(vary + (size_t) vref[i] * nw + k), iw[i]), w[i]));
				out[k] = __float_as_uint(__fmul_rn(v, recip));
			} else if (mode == kAffine || affineOnly) {
				float v = 0.0f;
#pragma unroll
				for (int i = 0; i < N; ++i)
					v = __fadd_rn(v, __fmul_rn(ldf(vary + (size_t) vref[i] * nw + k), w[i]));
				out[k] = __float_as_uint(v);
			} else {
				out[k] = vary[(size_t) vref[prov] * nw + k];
			}
		}
	}
}

/* General layouts (double, 1/2/8-byte integers, unaligned attributes): the
 * same rules, element by element on bytes. */
template <int N>
__device__ void interpolateBytes(const VaryingLayout& L, const uint32_t* vary, const uint32_t vref[N],
                                 const float w[N], const float iw[N], float recip, bool provFirst,
                                 bool affineOnly, uint32_t out[kMaxVaryingWords])
{
	const int prov = provFirst ? 0 : N - 1;
	const int nw = L.nWords;
	unsigned char* dst = (unsigned char*) out;
	for (int a = 0; a < L.nAttr; ++a) {
		const VaryingAttr at = L.attr[a];
		const unsigned char* src[N];
		for (int i = 0; i < N; ++i) src[i] = (const unsigned char*) (vary + (size_t) vref[i] * nw) + at.offset;
		const bool persp = at.mode == kPerspective && !affineOnly;
		const bool affine = at.mode == kAffine || affineOnly;
		if (at.type == SRP_FLOAT) {
			for (int e = 0; e < at.nItems; ++e) {
				float v = 0.0f;
				if (persp) {
					for (int i = 0; i < N; ++i) { float x; memcpy(&x, src[i] + 4 * e, 4); v = __fadd_rn(v, __fmul_rn(__fmul_rn(x, iw[i]), w[i])); }
					v = __fmul_rn(v, recip);
				} else if (affine) {
					for (int i = 0; i < N; ++i) { float x; memcpy(&x, src[i] + 4 * e, 4); v = __fadd_rn(v, __fmul_rn(x, w[i])); }
				} else memcpy(&v, src[prov] + 4 * e, 4);
				memcpy(dst + at.offset + 4 * e, &v, 4);
			}
		} else if (at.type == SRP_DOUBLE) {
			for (int e = 0; e < at.nItems; ++e) {
				double v = 0.0;
				if (persp) {
					for (int i = 0; i < N; ++i) { double x; memcpy(&x, src[i] + 8 * e, 8); v = __dadd_rn(v, __dmul_rn(__dmul_rn(x, (double) iw[i]), (double) w[i])); }
					v = __dmul_rn(v, (double) recip);
				} else if (affine) {
					for (int i = 0; i < N; ++i) { double x; memcpy(&x, src[i] + 8 * e, 8); v = __dadd_rn(v, __dmul_rn(x, (double) w[i])); }
				} else memcpy(&v, src[prov] + 8 * e, 8);
				memcpy(dst + at.offset + 8 * e, &v, 8);
			}
		} else {
			memcpy(dst + at.offset, src[prov], (size_t) at.elemSize * at.nItems);
		}
	}
}

template <int N>
__device__ __forceinline__ void interpolate(const VaryingLayout& L, const uint32_t* vary, const uint32_t vref[N],
                                            const float w[N], const float iw[N], float recip, bool provFirst,
                                            bool affineOnly, uint32_t out[kMaxVaryingWords])
{
	if (L.floatOnly) interpolateWords<N>(L, vary, vref, w, iw, recip, provFirst, affineOnly, out);
	else interpolateBytes<N>(L, vary, vref, w, iw, recip, provFirst, affineOnly, out);
}

/* ----------------------------------------------------- triangle helpers */

/* Barycentrics of triangle r at pixel (x, y): the exact serial chain
 * l0 -> (y - minY) row steps -> (x - minX) column steps. */
__device__ __forceinline__ void lambdaAt(const TriRaster& r, int x, int y, float l[3])
{
#pragma unroll
	for (int i = 0; i < 3; ++i)
		l[i] = srpChainAdd(srpChainAdd(r.l0[i], r.dy[i], (uint32_t) (y - r.minY)), r.dx[i], (uint32_t) (x - r.minX));
}

/* Top-left inside test; lambda[i] is paired with the flag of edge i
 * (src/raster/triangle.c:82-87, 153-157). */
__device__ __forceinline__ bool insideTri(const float l[3], uint32_t flags)
{
	bool in = true;
#pragma unroll
	for (int i = 0; i < 3; ++i)
		in = in && ((l[i] > 0.0f) || (roughlyZero(l[i]) && ((flags >> (1 + i)) & 1u)));
	return in;
}

/* depth = ((c0 l0 + c1 l1) + c2 l2) with c_i = z_ndc,i * invW_i
 * (src/pipeline/interpolation.c:34-47). */
__device__ __forceinline__ float triDepth(const float c[3], const float l[3])
{
	return __fadd_rn(__fadd_rn(__fmul_rn(c[0], l[0]), __fmul_rn(c[1], l[1])), __fmul_rn(c[2], l[2]));
}

__device__ __forceinline__ float triRecip(const float iw[3], const float l[3])
{
	return __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(__fmul_rn(iw[0], l[0]), __fmul_rn(iw[1], l[1])), __fmul_rn(iw[2], l[2])));
}

/* Bounded spin budget for waits on other blocks; a draw may set a smaller
 * one (DrawParams::spinLimit, 0 = this default). */
constexpr unsigned kSpinLimit = 1u << 24;
__device__ __forceinline__ unsigned spinBudget(uint32_t limit) { return limit ? limit : kSpinLimit; }

/* Decoupled look-back over a status array whose words hold a 2-bit flag in
 * the top bits (0 not yet published, 1 block aggregate, 2 inclusive prefix)
 * and a value below. Starting at predecessor j, returns the sum of values up
 * to and including the nearest inclusive prefix. W predecessors are loaded
 * per step with independent loads, so a block that has to walk far back (all
 * blocks of a wave finish their local work together) waits W times fewer
 * load latencies. A predecessor that has not published yet is re-read with
 * a bounded spin; on timeout the error bit is set and the walk ends. */
template <typename T, int W>
__device__ __forceinline__ T lookBack(const T* status, long long j, int flagShift, T valueMask, unsigned* errors,
                                      unsigned limit = kSpinLimit)
{
	T acc = 0;
	unsigned spins = 0;
	while (j >= 0) {
		T v[W];
#pragma unroll
		for (int k = 0; k < W; ++k)
			v[k] = (j - k >= 0) ? *((volatile const T*) (status + (j - k))) : ((T) 2 << flagShift);
#pragma unroll
		for (int k = 0; k < W; ++k) {
			while ((v[k] >> flagShift) == 0) {
				if (++spins > limit) { atomicOr(errors, kErrSpin); return acc; }
				__nanosleep(32);
				v[k] = *((volatile const T*) (status + (j - k)));
			}
			acc += v[k] & valueMask;
			if ((v[k] >> flagShift) == 2) return acc;
		}
		j -= W;
	}
	return acc;
}

}  // namespace srpg
