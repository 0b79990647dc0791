/* Device code shared by the per-tile kernels of k_raster.cu (visibility
 * resolve) and k_shade.cu (deferred and learned shading): the built-in
 * shaders, fragment inputs, item records and coverage, learned-shading
 * inputs, and where a tile lives (single draw or multi-draw pass). */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "kernels.h"
#include "launch.cuh"
#include "mlp.h"
#include "tc5.cuh"
#include "tma.cuh"
#include "srp/buffer.h"

namespace srpg {
__device__ __forceinline__ void rasterTexSample(const void* tex, float u, float v, float out[4])
{
	textureSample((const TextureDesc*) tex, u, v, out);
}
__device__ __forceinline__ void rasterTexSampleLod(const void* tex, float u, float v, float lod, float out[4])
{
	textureSampleLod((const TextureDesc*) tex, u, v, lod, out);
}
}  // namespace srpg
#define SRP_DEVICE_TEXTURE_SAMPLE(tex, u, v, out) srpg::rasterTexSample((const void*) (tex), u, v, out)
#define SRP_DEVICE_TEXTURE_SAMPLE_LOD(tex, u, v, lod, out) srpg::rasterTexSampleLod((const void*) (tex), u, v, lod, out)
#include "srp/shaderlib_impl.h"

namespace srpg {

constexpr int kResolveWarps = 4;
constexpr int kShadeTiles = 2;     /* tiles per block of k_shade (64 threads each) */
/* Light tiles of a multi-draw pass: items per chunk of a warp. Fewer than
 * the 32 lanes, so that the per-item depth rows take half the shared memory
 * and 8 blocks (64 registers a thread) fit an SM: the many light tiles of a
 * batch gain from the occupancy. Single draws keep chunks of 32 (measured
 * faster on the 1080p frame). */
constexpr int kResolveChunkMulti = 16;
/* row pitch of the per-item depth rows in shared memory: 65 keeps lanes that
 * write the same pixel of different items in different banks */
constexpr int kDepRow = 65;
constexpr int kHeavyThreads = 256;

template <int FS>
__device__ __forceinline__ void runFS(SRPFragmentShaderIn* in, SRPFragmentShaderOut* out)
{
	switch (FS) {
	case SRP_GPU_FS_VARYING_COLOR: srpslFsVaryingColor(in, out); break;
	case SRP_GPU_FS_SOLID: srpslFsSolid(in, out); break;
	case SRP_GPU_FS_PRIMITIVE_ID: srpslFsPrimitiveId(in, out); break;
	case SRP_GPU_FS_TEXTURE: srpslFsTexture(in, out); break;
	case SRP_GPU_FS_TEXTURE_MODULATE: srpslFsTextureModulate(in, out); break;
	case SRP_GPU_FS_BLINN_PHONG: srpslFsBlinnPhong(in, out); break;
	case SRP_GPU_FS_MARBLE: srpslFsMarble(in, out); break;
	case SRP_GPU_FS_DEPTH_OVERWRITE: srpslFsDepthOverwrite(in, out); break;
	case SRP_GPU_FS_FRAGCOORD: srpslFsFragCoord(in, out); break;
	case SRP_GPU_FS_FLAT_INT: srpslFsFlatInt(in, out); break;
	case SRP_GPU_FS_MIXED: srpslFsMixed(in, out); break;
	case SRP_GPU_FS_BYTE_PALETTE: srpslFsBytePalette(in, out); break;
	case SRP_GPU_FS_PRIMITIVE_MOD: srpslFsPrimitiveMod(in, out); break;
	case SRP_GPU_FS_TEXTURE_LOD: srpslFsTextureLod(in, out); break;
	default: break;
	}
}

/* Shader inputs of `item` at pixel (gx, gy): fragCoord and varyings as
 * built by src/raster/triangle.c:89-99, line.c:62-75, point.c:107-116.
 * The varyings go to `words`, which in.varyings points at. */
template <int KIND>
__device__ __forceinline__ void fragmentIn(const DrawParams& P, const unsigned char* uniform, uint32_t primBase,
                                           uint32_t item, int gx, int gy, SRPFragmentShaderIn& in, uint32_t* words)
{
	in.uniform = (SRPUniform*) uniform;
	in.varyings = (SRPInterpolated*) words;
	if (KIND == kKindTri) {
		const TriRaster R = P.triR[item];
		const TriAttr A = P.triA[item];
		float l[3];
		if (R.table != kNoTable) {
			/* table entry of this row and tile column, then the remaining steps */
			const int ncols = ((int) R.maxX - 1) / kTile - (int) R.minX / kTile + 1;
			const int col = gx / kTile;
			const float* T = P.table + R.table + 3 * ((size_t) (gy - R.minY) * ncols + (col - (int) R.minX / kTile));
			const int xs = max((int) R.minX, col * kTile);
#pragma unroll
			for (int i = 0; i < 3; ++i) {
				float v = T[i];
				for (int x = xs; x < gx; ++x) v = __fadd_rn(v, R.dx[i]);
				l[i] = v;
			}
		} else {
			lambdaAt(R, gx, gy, l);
		}
		const float depth = triDepth(R.c, l);
		const float recip = triRecip(A.invW, l);
		interpolate<3>(P.L, P.vary, A.vref, l, A.invW, recip, P.st.provokingFirst, false, words);
		in.fragCoord[0] = __fadd_rn((float) gx, 0.5f);
		in.fragCoord[1] = __fadd_rn((float) gy, 0.5f);
		in.fragCoord[2] = depth;
		in.fragCoord[3] = recip;
		in.frontFacing = (R.flags & 1u) != 0;
		in.primitiveID = A.id - primBase;
	} else if (KIND == kKindLineFrag) {
		const LineFrag F = P.frags[item];
		const LineRec L = P.lines[F.line];
		const float w[2] = { __fsub_rn(1.0f, F.t), F.t };
		const float recip = __fdiv_rn(1.0f, __fadd_rn(__fmul_rn(L.invW[0], w[0]), __fmul_rn(L.invW[1], w[1])));
		interpolate<2>(P.L, P.vary, L.vref, w, L.invW, recip, P.st.provokingFirst, false, words);
		in.fragCoord[0] = __fadd_rn((float) F.px, 0.5f);
		in.fragCoord[1] = __fadd_rn((float) F.py, 0.5f);
		in.fragCoord[2] = F.depth;
		in.fragCoord[3] = recip;
		in.frontFacing = true;
		in.primitiveID = L.id;
	} else {
		const PointRec R = P.points[item];
		const int nw = P.L.nWords;
#pragma unroll
		for (int k = 0; k < kMaxVaryingWords; ++k)
			if (k < nw) words[k] = P.vary[(size_t) R.vref * nw + k];
		in.fragCoord[0] = __fadd_rn((float) gx, 0.5f);
		in.fragCoord[1] = __fadd_rn((float) gy, 0.5f);
		in.fragCoord[2] = R.z;
		in.fragCoord[3] = 1.0f;
		in.frontFacing = true;
		in.primitiveID = R.id;
	}
}

template <int FS>
__device__ __forceinline__ void runShader(SRPFragmentShaderIn& in, SRPFragmentShaderOut& out)
{
	out.color[0] = out.color[1] = out.color[2] = out.color[3] = 0.0f;
	out.fragDepth = __int_as_float(0x7FC00000);
	runFS<FS>(&in, &out);
}

/* The shader call for `item` at pixel (gx, gy). */
template <int KIND, int FS>
__device__ __forceinline__ void shadeItem(const DrawParams& P, const unsigned char* uniform, uint32_t primBase,
                                          uint32_t item, int gx, int gy, SRPFragmentShaderOut& out)
{
	uint32_t words[kMaxVaryingWords];
	SRPFragmentShaderIn in;
	fragmentIn<KIND>(P, uniform, primBase, item, gx, gy, in, words);
	runShader<FS>(in, out);
}

/* The pixel a line fragment lands on, as the reference indexes it: its
 * logical (px, py) when 0 <= px < W and py >= 0; otherwise the row-major
 * index py * W + px wraps (px may equal the width), and the pixel comes
 * from it. */
__device__ __forceinline__ void lineFragPixel(int W, int px, int py, int& gx, int& gy)
{
	if ((unsigned) px < (unsigned) W && py >= 0) { gx = px; gy = py; return; }
	const unsigned long long at = (unsigned long long) (long long) py * (unsigned long long) W
	                            + (unsigned long long) (long long) px;
	gx = (int) (at % (unsigned long long) W);
	gy = (int) (at / (unsigned long long) W);
}

/* Record of an item, by kind (loaded ahead of use by k_resolve_heavy). */
template <int KIND> struct RecOf { typedef TriRaster T; };
template <> struct RecOf<kKindPoint> { typedef PointRec T; };
template <> struct RecOf<kKindLineFrag> { typedef LineFrag T; };

template <int KIND>
__device__ __forceinline__ typename RecOf<KIND>::T loadRec(const DrawParams& P, uint32_t item)
{
	if constexpr (KIND == kKindTri) return P.triR[item];
	else if constexpr (KIND == kKindPoint) return P.points[item];
	else return P.frags[item];
}

/* Phase 1: coverage of one item (its record) over the tile at (x0, y0). */
template <int KIND>
__device__ __forceinline__ void coverageRec(const DrawParams& P, const typename RecOf<KIND>::T& Rec, int x0, int y0,
                                            unsigned long long& mask, float* dep, uint32_t& flags)
{
	mask = 0;
	if constexpr (KIND == kKindTri) {
		const TriRaster& R = Rec;
		flags = R.flags;
		const int xs = max(x0, (int) R.minX), xe = min(x0 + kTile, (int) R.maxX);
		const int ys = max(y0, (int) R.minY), ye = min(y0 + kTile, (int) R.maxY);
		if (xs >= xe || ys >= ye) return;
		/* row starts: the big-triangle table, or the exact chain */
		const float* T = nullptr;
		int ncols = 0;
		if (R.table != kNoTable) {
			ncols = ((int) R.maxX - 1) / kTile - (int) R.minX / kTile + 1;
			T = P.table + R.table + 3 * ((size_t) (ys - R.minY) * ncols + (x0 / kTile - (int) R.minX / kTile));
		}
		float lr[3];
		if (!T) {
#pragma unroll
			for (int i = 0; i < 3; ++i) lr[i] = srpChainAdd(R.l0[i], R.dy[i], (uint32_t) (ys - R.minY));
		}
		for (int y = ys; y < ye; ++y) {
			float l[3];
			if (T) {
#pragma unroll
				for (int i = 0; i < 3; ++i) l[i] = T[i];
				T += 3 * ncols;
			} else {
#pragma unroll
				for (int i = 0; i < 3; ++i) l[i] = srpChainAdd(lr[i], R.dx[i], (uint32_t) (xs - R.minX));
			}
			for (int x = xs; x < xe; ++x) {
				if (insideTri(l, R.flags)) {
					const int q = (y - y0) * kTile + (x - x0);
					mask |= 1ull << q;
					dep[q] = triDepth(R.c, l);
				}
#pragma unroll
				for (int i = 0; i < 3; ++i) l[i] = __fadd_rn(l[i], R.dx[i]);
			}
			if (!T) {
#pragma unroll
				for (int i = 0; i < 3; ++i) lr[i] = __fadd_rn(lr[i], R.dy[i]);
			}
		}
	} else if constexpr (KIND == kKindPoint) {
		const PointRec& R = Rec;
		flags = 1u;
		const int xs = max(x0, (int) R.x0), xe = min(x0 + kTile - 1, (int) R.x1);
		const int ys = max(y0, (int) R.y0), ye = min(y0 + kTile - 1, (int) R.y1);
		for (int y = ys; y <= ye; ++y)
			for (int x = xs; x <= xe; ++x) {
				const float cx = __fadd_rn((float) x, 0.5f), cy = __fadd_rn((float) y, 0.5f);
				if (cx < R.mnx || cx >= R.mxx || cy < R.mny || cy >= R.mxy) continue;
				const int q = (y - y0) * kTile + (x - x0);
				mask |= 1ull << q;
				dep[q] = R.z;
			}
	} else {
		const LineFrag& F = Rec;
		flags = 1u;
		int gx, gy;
		lineFragPixel(P.st.W, F.px, F.py, gx, gy);
		const int q = (gy - y0) * kTile + (gx - x0);
		if (q >= 0 && q < 64) { mask = 1ull << q; dep[q] = F.depth; }
	}
}

template <int KIND>
__device__ __forceinline__ void coverage(const DrawParams& P, uint32_t item, int x0, int y0,
                                         unsigned long long& mask, float* dep, uint32_t& flags)
{
	coverageRec<KIND>(P, loadRec<KIND>(P, item), x0, y0, mask, dep, flags);
}

/* Tile-relative span of triangle R over the tile at (x0, y0): columns
 * [xs, xe), first row ys, packed 4 bits each; returns the number of rows. */
__device__ __forceinline__ uint32_t triSpan(const TriRaster& R, int x0, int y0, uint32_t& span)
{
	const int xs = max(x0, (int) R.minX), xe = min(x0 + kTile, (int) R.maxX);
	const int ys = max(y0, (int) R.minY), ye = min(y0 + kTile, (int) R.maxY);
	span = 0;
	if (xs >= xe || ys >= ye) return 0;
	span = (uint32_t) (xs - x0) | (uint32_t) (xe - x0) << 4 | (uint32_t) (ys - y0) << 8;
	return (uint32_t) (ye - ys);
}

/* One row of a triangle inside a tile: barycentrics at the first column
 * (big-triangle table, or the exact chain l0 -> row -> column), then the
 * reference's per-pixel steps. Sets the covered bits and stores the depths. */
__device__ __forceinline__ unsigned long long triRow(const DrawParams& P, const TriRaster& R, int x0, int y0, int xs,
                                                     int xe, int y, float* dep)
{
	float l[3];
	if (R.table != kNoTable) {
		const int ncols = ((int) R.maxX - 1) / kTile - (int) R.minX / kTile + 1;
		const float* T = P.table + R.table + 3 * ((size_t) (y - R.minY) * ncols + (x0 / kTile - (int) R.minX / kTile));
		l[0] = T[0]; l[1] = T[1]; l[2] = T[2];
	} else {
#pragma unroll
		for (int i = 0; i < 3; ++i)
			l[i] = srpChainAdd(srpChainAdd(R.l0[i], R.dy[i], (uint32_t) (y - R.minY)), R.dx[i], (uint32_t) (xs - R.minX));
	}
	unsigned long long bits = 0;
	for (int x = xs; x < xe; ++x) {
		if (insideTri(l, R.flags)) {
			const int q = (y - y0) * kTile + (x - x0);
			bits |= 1ull << q;
			dep[q] = triDepth(R.c, l);
		}
#pragma unroll
		for (int i = 0; i < 3; ++i) l[i] = __fadd_rn(l[i], R.dx[i]);
	}
	return bits;
}

/* Index of the item owning flattened row p: the last j with off[j] <= p
 * (items without rows share their successor's offset and are skipped). */
template <int N>
__device__ __forceinline__ int findOwner(const uint32_t* off, uint32_t p)
{
	int lo = 0, hi = N;
	while (hi - lo > 1) {
		const int mid = (lo + hi) >> 1;
		if (off[mid] <= p) lo = mid; else hi = mid;
	}
	return lo;
}

/* ------------------------------------------------------ learned shading */

__device__ __forceinline__ float clamp01f(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

/* 1 pixel in `every`, by a hash of the pixel and a seed. */
__device__ __forceinline__ bool pixelSampled(int gx, int gy, uint32_t seed, uint32_t every)
{
	if (every <= 1) return every == 1;
	uint32_t h = (uint32_t) gx * 0x9E3779B1u ^ (uint32_t) gy * 0x85EBCA77u ^ seed * 0xC2B2AE3Du;
	h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
	return h % every == 0;
}

/* The learned network's inputs at a fragment: world position and normal
 * (varyings 0..5 of srpVsWorld), the normal normalised and the view direction
 * towards the uniform's camera, as the lighting shaders compute them. */
__device__ __forceinline__ void learnedInputs(const unsigned char* uniform, const uint32_t* words, float* x9)
{
	const SRPStdUniform* u = (const SRPStdUniform*) uniform;
	float n[3], v[3];
	for (int k = 0; k < 3; ++k) {
		x9[k] = __uint_as_float(words[k]);
		n[k] = __uint_as_float(words[3 + k]);
		v[k] = u->cameraPos[k] - x9[k];
	}
	srpslNormalize3(n);
	srpslNormalize3(v);
	for (int k = 0; k < 3; ++k) { x9[3 + k] = n[k]; x9[6 + k] = v[k]; }
}

__device__ __forceinline__ void captureSample(const DrawParams& P, const unsigned char* uniform, const uint32_t* words,
                              const SRPFragmentShaderOut& out)
{
	const unsigned long long slot = atomicAdd(P.captureCount, 1ull);
	if (slot >= P.captureCap) return;
	float* s = P.capture + slot * kSampleFloats;
	learnedInputs(uniform, words, s);
	for (int k = 0; k < 3; ++k) s[9 + k] = clamp01f(out.color[k]);
}

/* Where a tile's pixels live: its origin in its framebuffer, the
 * framebuffer's size and planes, and the uniform and primitive-id base of
 * its draw. A single draw takes them from the parameters; a multi-draw pass
 * (MULTI) from the descriptor of the draw the global tile belongs to. */
struct TileCtx {
	uint32_t d;          /* draw of the tile (0 for a single draw) */
	int x0, y0, W, H;
	uint32_t* color;
	float* depth;
	uint8_t* stencil;
	int32_t* winner;
	const unsigned char* uniform;
	uint32_t primBase;
};

__device__ __forceinline__ uint32_t tileDraw(const uint32_t* prefix, uint32_t n, uint32_t x)
{
	uint32_t lo = 0, hi = n;
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (__ldg(prefix + mid) <= x) lo = mid; else hi = mid;
	}
	return lo;
}

template <bool MULTI>
__device__ __forceinline__ TileCtx tileCtx(const DrawParams& P, uint32_t tile)
{
	TileCtx c;
	if constexpr (MULTI) {
		const uint32_t d = tileDraw(P.tPrefix, P.nDraws, tile);
		const DrawDesc& D = P.draws[d];
		const uint32_t lt = tile - P.tPrefix[d];
		c.d = d;
		c.x0 = (int) (lt % (uint32_t) D.tilesX) * kTile;
		c.y0 = (int) (lt / (uint32_t) D.tilesX) * kTile;
		c.W = D.W; c.H = D.H;
		c.color = D.color; c.depth = D.depth; c.stencil = D.stencil; c.winner = D.winner;
		c.uniform = D.uniform;
		c.primBase = P.primPrefix[d];
	} else {
		c.d = 0;
		c.x0 = (int) (tile % (uint32_t) P.st.tilesX) * kTile;
		c.y0 = (int) (tile / (uint32_t) P.st.tilesX) * kTile;
		c.W = P.st.W; c.H = P.st.H;
		c.color = P.color; c.depth = P.depth; c.stencil = P.stencil; c.winner = P.winner;
		c.uniform = P.uniform;
		c.primBase = 0;
	}
	return c;
}

/* LATE_FS = 0: early depth test, colour deferred to k_shade.
 * LATE_FS = a fragment shader id: the shader runs per fragment in order and
 * may replace the depth (src/raster/fragment.c:97-111). */
}  // namespace srpg
