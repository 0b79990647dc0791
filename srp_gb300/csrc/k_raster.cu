/* Per-tile rasterisation: visibility resolve and deferred shading.
 *
 * One warp owns one 8x8 tile; lane l owns pixels l and l + 32 of it. The
 * tile's items (triangles, points or line fragments, already in submission
 * order) are taken 32 at a time:
 *   phase 1  lane j evaluates item j over the tile -- for a triangle the
 *            reference's incremental barycentrics (exact chain, see chain.h)
 *            and the top-left test -- leaving a 64-bit coverage mask and the
 *            per-pixel depths in shared memory;
 *   phase 2  each lane walks, for its own pixels, the covering items in order
 *            and applies the stencil test, the depth test and the stencil
 *            operations exactly as the reference's emitFragment does
 *            (src/raster/fragment.c:63-125), remembering the last item that
 *            reached the colour write.
 * Because srp has no blending and a shader that does not write fragDepth
 * cannot influence depth or stencil, the colour of a pixel is the shader
 * output of that last item; k_shade evaluates it once per pixel afterwards.
 * Shaders that write fragDepth take the in-order path (k_resolve with
 * LATE_FS), which shades every fragment in phase 2. */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "kernels.h"
#include "launch.cuh"
#include "mlp.h"
#include "tc5.cuh"
#include "srp/buffer.h"

namespace srpg {
__device__ __forceinline__ void rasterTexSample(const void* tex, float u, float v, float out[4])
{
	textureSample((const TextureDesc*) tex, u, v, out);
}
}  // namespace srpg
#define SRP_DEVICE_TEXTURE_SAMPLE(tex, u, v, out) srpg::rasterTexSample((const void*) (tex), u, v, out)
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
		const unsigned long long idx = (unsigned long long) (long long) F.py * (unsigned long long) P.st.W
		                             + (unsigned long long) (long long) F.px;
		const int gx = (int) (idx % (unsigned long long) P.st.W), gy = (int) (idx / (unsigned long long) P.st.W);
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

__device__ void captureSample(const DrawParams& P, const unsigned char* uniform, const uint32_t* words,
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
template <int KIND, int LATE_FS, bool MULTI = false>
__global__ void __launch_bounds__(kResolveWarps * 32, MULTI ? 8 : 1) k_resolve(const __grid_constant__ DrawParams P,
                                                                              const uint32_t* vals, uint32_t numTiles)
{
	gridDepSync();
	constexpr int kResolveChunk = MULTI ? kResolveChunkMulti : 32;
	__shared__ unsigned long long sMask[kResolveWarps][32];
	__shared__ uint32_t sItem[kResolveWarps][32];
	__shared__ uint32_t sFlag[kResolveWarps][32];
	__shared__ float sDep[kResolveWarps][kResolveChunk][kDepRow];
	__shared__ TriRaster sRec[KIND == kKindTri ? kResolveWarps : 1][kResolveChunk];
	__shared__ uint32_t sOff[kResolveWarps][32];
	__shared__ uint32_t sSpan[kResolveWarps][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t tile = blockIdx.x * kResolveWarps + warp;
	if (tile >= numTiles || P.ctr->abort) return;
	const uint32_t s = P.tileStart[tile], e = P.tileEnd[tile];
	if (s >= e) return;
	if (LATE_FS == 0 && e - s > P.heavyItems) return;  /* k_resolve_heavy's */
	const DrawState& st = P.st;
	const TileCtx c = tileCtx<MULTI>(P, tile);
	const int x0 = c.x0, y0 = c.y0;

	float depth[2];
	uint32_t sten[2], col[2];
	int32_t win[2];
	bool ok[2];
	size_t idx[2];
	int gx[2], gy[2];
#pragma unroll
	for (int p = 0; p < 2; ++p) {
		const int q = lane + 32 * p;
		gx[p] = x0 + (q & 7);
		gy[p] = y0 + (q >> 3);
		const bool valid = gx[p] < c.W && gy[p] < c.H;
		idx[p] = valid ? (size_t) gy[p] * c.W + gx[p] : 0;
		depth[p] = valid ? c.depth[idx[p]] : 0.0f;
		sten[p] = valid ? c.stencil[idx[p]] : 0u;
		col[p] = 0;
		win[p] = -1;
		/* line fragments were scissor-tested on their logical coordinates */
		ok[p] = valid && (KIND == kKindLineFrag || scissorPass(st, gx[p], gy[p]));
	}
	unsigned long long frags = 0;
	for (uint32_t b = s; b < e; b += kResolveChunk) {
		const uint32_t n = min((uint32_t) kResolveChunk, e - b);
		unsigned long long mask = 0;
		uint32_t item = 0, flags = 0;
		if (KIND == kKindTri) {
			/* triangles: coverage over flattened (item, row) pairs so that the
			 * lanes share the work whatever the items' sizes */
			uint32_t rows = 0, span = 0;
			if ((uint32_t) lane < n) {
				item = vals[b + lane];
				const TriRaster R = P.triR[item];
				sRec[warp][lane] = R;
				flags = R.flags;
				rows = triSpan(R, x0, y0, span);
			}
			uint32_t incl = rows;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
				if (lane >= o) incl += y;
			}
			const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
			sOff[warp][lane] = incl - rows;
			sSpan[warp][lane] = span;
			sMask[warp][lane] = 0;
			__syncwarp();
			for (uint32_t pr = lane; pr < total; pr += 32) {
				const int j = findOwner<32>(sOff[warp], pr);
				const uint32_t sp = sSpan[warp][j];
				const int xs = x0 + (int) (sp & 15u), xe = x0 + (int) ((sp >> 4) & 15u);
				const int y = y0 + (int) ((sp >> 8) & 15u) + (int) (pr - sOff[warp][j]);
				const unsigned long long bits = triRow(P, sRec[warp][j], x0, y0, xs, xe, y, sDep[warp][j]);
				if (bits) atomicOr(&sMask[warp][j], bits);
			}
			__syncwarp();
		} else {
			if ((uint32_t) lane < n) {
				item = vals[b + lane];
				coverage<KIND>(P, item, x0, y0, mask, sDep[warp][lane], flags);
			}
			sMask[warp][lane] = mask;
		}
		sItem[warp][lane] = item;
		sFlag[warp][lane] = flags;
		__syncwarp();
#pragma unroll
		for (int p = 0; p < 2; ++p) {
			if (!ok[p]) continue;
			const int q = lane + 32 * p;
			uint32_t m = 0;
			for (uint32_t j = 0; j < n; ++j) m |= (uint32_t) ((sMask[warp][j] >> q) & 1ull) << j;
			frags += __popc(m);
			while (m) {
				const int j = __ffs(m) - 1;
				m &= m - 1;
				const bool front = (sFlag[warp][j] & 1u) != 0;
				const StencilFace& sf = front ? st.front : st.back;
				float d = sDep[warp][j][q];
				if (st.stencilEnabled && !stencilCompare(sf.ref, sten[p], sf.mask, sf.func)) {
					sten[p] = stencilApply(sf.sfail, sten[p], sf.ref, sf.writeMask);
					continue;
				}
				if (LATE_FS == 0) {
					if (st.depthTest && !depthCompare(st.depthOp, d, depth[p])) {
						if (st.stencilEnabled) sten[p] = stencilApply(sf.dfail, sten[p], sf.ref, sf.writeMask);
						continue;
					}
				} else {
					SRPFragmentShaderOut out;
					shadeItem<KIND, LATE_FS>(P, c.uniform, c.primBase, sItem[warp][j], gx[p], gy[p], out);
					if (!isnan(out.fragDepth)) d = out.fragDepth;
					if (st.depthTest && !depthCompare(st.depthOp, d, depth[p])) {
						if (st.stencilEnabled) sten[p] = stencilApply(sf.dfail, sten[p], sf.ref, sf.writeMask);
						continue;
					}
					col[p] = packColor(out.color);
				}
				if (st.stencilEnabled) sten[p] = stencilApply(sf.pass, sten[p], sf.ref, sf.writeMask);
				win[p] = (int32_t) sItem[warp][j];
				if (st.depthTest && st.depthWrite) depth[p] = d;
			}
		}
		__syncwarp();
	}
#pragma unroll
	for (int p = 0; p < 2; ++p) {
		if (!(gx[p] < c.W && gy[p] < c.H)) continue;
		c.depth[idx[p]] = depth[p];
		c.stencil[idx[p]] = (uint8_t) sten[p];
		if (LATE_FS == 0) c.winner[idx[p]] = win[p];
		else if (win[p] >= 0) c.color[idx[p]] = col[p];
	}
	if (KIND != kKindLineFrag) {
		for (int o = 16; o; o >>= 1) frags += __shfl_xor_sync(0xFFFFFFFFu, frags, o);
		if (lane == 0 && frags) atomicAdd(&P.ctr->fragments, frags);
	}
}

/* Applies one fragment to a pixel's depth/stencil state (early depth test;
 * src/raster/fragment.c:63-125). Returns true if it reached the colour write. */
__device__ __forceinline__ bool applyFragment(const DrawState& st, bool front, float d, float& depth, uint32_t& sten)
{
	const StencilFace& sf = front ? st.front : st.back;
	if (st.stencilEnabled && !stencilCompare(sf.ref, sten, sf.mask, sf.func)) {
		sten = stencilApply(sf.sfail, sten, sf.ref, sf.writeMask);
		return false;
	}
	if (st.depthTest && !depthCompare(st.depthOp, d, depth)) {
		if (st.stencilEnabled) sten = stencilApply(sf.dfail, sten, sf.ref, sf.writeMask);
		return false;
	}
	if (st.stencilEnabled) sten = stencilApply(sf.pass, sten, sf.ref, sf.writeMask);
	if (st.depthTest && st.depthWrite) depth = d;
	return true;
}

/* Light tiles of line fragments (early depth test). Every item is one
 * fragment on one pixel, so no coverage masks are needed: a warp takes 32
 * fragments at a time, the lanes whose fragments land on the same pixel find
 * each other with match.any, and the first of them applies the group's
 * fragments in item order to that pixel's depth/stencil state, which the
 * warp keeps in shared memory for the whole tile. */
__global__ void __launch_bounds__(kResolveWarps * 32) k_resolve_frags(const __grid_constant__ DrawParams P,
                                                                     const uint32_t* vals, uint32_t numTiles)
{
	gridDepSync();
	__shared__ float sDepth[kResolveWarps][64];
	__shared__ uint32_t sSten[kResolveWarps][64];
	__shared__ int32_t sWin[kResolveWarps][64];
	__shared__ float sFd[kResolveWarps][32];
	__shared__ uint32_t sFi[kResolveWarps][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t tile = blockIdx.x * kResolveWarps + warp;
	if (tile >= numTiles || P.ctr->abort) return;
	const uint32_t s = P.tileStart[tile], e = P.tileEnd[tile];
	if (s >= e || e - s > P.heavyItems) return;  /* empty, or k_resolve_heavy's */
	const DrawState& st = P.st;
	const TileCtx c = tileCtx<false>(P, tile);
	const int x0 = c.x0, y0 = c.y0;
	size_t idx[2];
	bool valid[2];
#pragma unroll
	for (int p = 0; p < 2; ++p) {
		const int q = lane + 32 * p;
		const int gx = x0 + (q & 7), gy = y0 + (q >> 3);
		valid[p] = gx < c.W && gy < c.H;
		idx[p] = valid[p] ? (size_t) gy * c.W + gx : 0;
		sDepth[warp][q] = valid[p] ? c.depth[idx[p]] : 0.0f;
		sSten[warp][q] = valid[p] ? c.stencil[idx[p]] : 0u;
		sWin[warp][q] = -1;
	}
	__syncwarp();
	for (uint32_t b = s; b < e; b += 32) {
		const uint32_t n = min(32u, e - b);
		int q = -1;
		float d = 0.0f;
		uint32_t item = 0;
		if ((uint32_t) lane < n) {
			item = vals[b + lane];
			const LineFrag F = P.frags[item];
			/* the logical pixel, as the reference indexes it (px may equal the width) */
			const unsigned long long at = (unsigned long long) (long long) F.py * (unsigned long long) st.W
			                            + (unsigned long long) (long long) F.px;
			const int gx = (int) (at % (unsigned long long) st.W), gy = (int) (at / (unsigned long long) st.W);
			const int qq = (gy - y0) * kTile + (gx - x0);
			if (qq >= 0 && qq < 64) q = qq;
			d = F.depth;
		}
		sFd[warp][lane] = d;
		sFi[warp][lane] = item;
		const unsigned peers = __match_any_sync(0xFFFFFFFFu, q);
		__syncwarp();
		if (q >= 0 && lane == __ffs(peers) - 1) {
			float depth = sDepth[warp][q];
			uint32_t sten = sSten[warp][q];
			int32_t win = sWin[warp][q];
			for (unsigned m = peers; m; m &= m - 1) {
				const int j = __ffs(m) - 1;
				if (applyFragment(st, true, sFd[warp][j], depth, sten)) win = (int32_t) sFi[warp][j];
			}
			sDepth[warp][q] = depth;
			sSten[warp][q] = sten;
			sWin[warp][q] = win;
		}
		__syncwarp();
	}
#pragma unroll
	for (int p = 0; p < 2; ++p) {
		if (!valid[p]) continue;
		const int q = lane + 32 * p;
		c.depth[idx[p]] = sDepth[warp][q];
		c.stencil[idx[p]] = (uint8_t) sSten[warp][q];
		c.winner[idx[p]] = sWin[warp][q];
	}
}

/* Tiles with many items (typically far-away meshes whose thousands of tiny
 * triangles land in a handful of tiles): a CTA takes 256 consecutive items
 * at a time, every thread evaluates one item's coverage and depths, warp
 * ballots transpose the coverage into per-pixel item masks, and 64 pixel
 * owners then apply just the covering fragments, in item order. Work per
 * chunk is parallel over items; per pixel only real fragments are walked.
 * Heavy tiles come from a list built by k_tile_classify and are pulled by a
 * fixed grid of CTAs. */
template <int KIND, bool MULTI = false>
__global__ void __launch_bounds__(kHeavyThreads) k_resolve_heavy(const __grid_constant__ DrawParams P,
                                                                const uint32_t* vals, const uint32_t* heavy)
{
	gridDepSync();
	extern __shared__ float hDep[];                 /* [kHeavyThreads][kDepRow] */
	__shared__ uint32_t ballots[kHeavyThreads / 32][64];
	__shared__ uint32_t hFlag[kHeavyThreads], hItem[kHeavyThreads];

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const DrawState& st = P.st;
	const uint32_t nHeavy = P.ctr->abort ? 0u : P.ctr->nonEmptyTiles;
	for (uint32_t h = blockIdx.x; h < nHeavy; h += gridDim.x) {
		const uint32_t tile = heavy[h];
		const uint32_t s = P.tileStart[tile], e = P.tileEnd[tile];
		const TileCtx c = tileCtx<MULTI>(P, tile);
		const int x0 = c.x0, y0 = c.y0;
		const int gx = x0 + (tid & 7), gy = y0 + ((tid >> 3) & 7);
		const bool owner = tid < 64;
		const bool valid = owner && gx < c.W && gy < c.H;
		const size_t idx = valid ? (size_t) gy * c.W + gx : 0;
		float depth = valid ? c.depth[idx] : 0.0f;
		uint32_t sten = valid ? c.stencil[idx] : 0u;
		int32_t win = -1;
		const bool ok = valid && (KIND == kKindLineFrag || scissorPass(st, gx, gy));
		unsigned long long frags = 0;
		uint32_t curItem = 0;
		typename RecOf<KIND>::T cur = {};
		if (s + tid < e) { curItem = vals[s + tid]; cur = loadRec<KIND>(P, curItem); }
		for (uint32_t b = s; b < e; b += kHeavyThreads) {
			const uint32_t n = min((uint32_t) kHeavyThreads, e - b);
			unsigned long long mask = 0;
			uint32_t item = 0, flags = 0;
			if ((uint32_t) tid < n) {
				item = curItem;
				coverageRec<KIND>(P, cur, x0, y0, mask, hDep + tid * kDepRow, flags);
			}
			/* prefetch the next chunk's item while this one is resolved */
			if (b + kHeavyThreads + tid < e) {
				curItem = vals[b + kHeavyThreads + tid];
				cur = loadRec<KIND>(P, curItem);
			}
			hFlag[tid] = flags;
			hItem[tid] = item;
			uint32_t lo = 0, hi = 0;
#pragma unroll
			for (int q = 0; q < 64; ++q) {
				const uint32_t bq = __ballot_sync(0xFFFFFFFFu, (mask >> q) & 1ull);
				if (lane == (q & 31)) { if (q < 32) lo = bq; else hi = bq; }
			}
			ballots[warp][lane] = lo;
			ballots[warp][32 + lane] = hi;
			__syncthreads();
			if (ok) {
				const int q = tid;
				for (int w = 0; w < kHeavyThreads / 32; ++w) {
					uint32_t m = ballots[w][q];
					frags += __popc(m);
					while (m) {
						const int j = w * 32 + __ffs(m) - 1;
						m &= m - 1;
						if (applyFragment(st, (hFlag[j] & 1u) != 0, hDep[j * kDepRow + q], depth, sten))
							win = (int32_t) hItem[j];
					}
				}
			}
			__syncthreads();
		}
		if (valid) {
			c.depth[idx] = depth;
			c.stencil[idx] = (uint8_t) sten;
			c.winner[idx] = win;
		}
		if (KIND != kKindLineFrag && warp < 2) {
			for (int o = 16; o; o >>= 1) frags += __shfl_xor_sync(0xFFFFFFFFu, frags, o);
			if (lane == 0 && frags) atomicAdd(&P.ctr->fragments, frags);
		}
	}
}

/* Lists the tiles with more than P.heavyItems items for k_resolve_heavy. */
__global__ void k_tile_classify(const __grid_constant__ DrawParams P, uint32_t numTiles, uint32_t* heavy)
{
	gridDepSync();
	const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= numTiles || P.ctr->abort) return;
	const uint32_t n = P.tileEnd[t] - P.tileStart[t];
	if (P.tileEnd[t] > P.tileStart[t] && n > P.heavyItems) heavy[atomicAdd(&P.ctr->nonEmptyTiles, 1u)] = t;
}

/* Deferred shading: one shader invocation per pixel whose colour was written
 * by the resolve pass. */
template <int KIND, int FS, bool MULTI = false>
__global__ void __launch_bounds__(kShadeTiles * 64) k_shade(const __grid_constant__ DrawParams P, uint32_t numTiles)
{
	gridDepSync();
	/* one pixel a thread, two warps a tile */
	const uint32_t tile = blockIdx.x * kShadeTiles + (threadIdx.x >> 6);
	const int q = threadIdx.x & 63;
	if (tile >= numTiles || P.ctr->abort) return;
	if (P.tileStart[tile] >= P.tileEnd[tile]) return;
	const TileCtx c = tileCtx<MULTI>(P, tile);
	if (MULTI && P.redo && !P.redo[c.d]) return;
	const int x0 = c.x0, y0 = c.y0;
	{
		const int gx = x0 + (q & 7), gy = y0 + (q >> 3);
		if (gx >= c.W || gy >= c.H) return;
		const size_t idx = (size_t) gy * c.W + gx;
		const int32_t w = c.winner[idx];
		if (w < 0) return;
		SRPFragmentShaderOut out;
		if constexpr (KIND == kKindTri && FS == SRP_GPU_FS_MARBLE) {
			/* the shader learned shading stands in for: captured for training */
			uint32_t words[kMaxVaryingWords];
			SRPFragmentShaderIn in;
			fragmentIn<KIND>(P, c.uniform, c.primBase, (uint32_t) w, gx, gy, in, words);
			runShader<FS>(in, out);
			if (P.capture && pixelSampled(gx, gy, P.sampleSeed + c.d, P.captureEvery))
				captureSample(P, c.uniform, words, out);
		} else {
			shadeItem<KIND, FS>(P, c.uniform, c.primBase, (uint32_t) w, gx, gy, out);
		}
		c.color[idx] = packColor(out.color);
	}
}

/* Learned shading on tcgen05. A CTA holds kLearnGroups independent groups of
 * 4 warps that share one copy of the weights in shared memory; each group
 * shades a pair of tiles (128 pixels, one per thread) at a time as one
 * 128-row MMA tile, with its own A tile, 64 TMEM columns, mbarrier and named
 * barrier, so that one group's fragment loads and encoding overlap another
 * group's MMA chain. Groups take the tile pairs in order from a counter of
 * the draw, one at a time, so that the CTAs end together. In a group each thread builds its pixel's encoded inputs
 * as row `gt` of the A tile; one thread issues each layer's MMAs into a
 * 128 x 64 fp32 accumulator in tensor memory; each warp reads its 32 lanes
 * (rows) back, adds the bias, applies ReLU and writes the next A tile, and
 * finally its pixels' colours. The judge runs afterwards as its own pass
 * (k_judge_learned). Every wait is bounded; on a timeout the group records
 * kErrSpin and stops, and the CTA releases its tensor memory and returns. */
constexpr int kLearnGroups = 6;
constexpr int kLearnThreads = 128 * kLearnGroups;
constexpr uint32_t kLearnCols = 512;   /* kLearnGroups x 64 columns, rounded up to a power of two */
constexpr size_t kLearnSmem = kTcWBytes + (size_t) kLearnGroups * kTcABytes + 208 * 4 + kLearnGroups * 8 + 16 +
                              kLearnGroups * 4;
static_assert(kLearnGroups * 64 <= (int) kLearnCols && kLearnCols <= 512, "TMEM columns");
static_assert(kLearnSmem <= 227 * 1024, "shared memory");

template <int KIND, bool MULTI>
__global__ void __launch_bounds__(kLearnThreads, 1) k_shade_learned5(const __grid_constant__ DrawParams P, uint32_t numTiles)
{
	gridDepSync();
	extern __shared__ __align__(1024) uint8_t tsm[];
	const int tid = threadIdx.x, warp = tid >> 5;
	const int g = warp >> 2, gt = tid & 127;          /* group, thread within the group */
	const uint32_t bar = 1u + (uint32_t) g;            /* the group's named barrier (0 is __syncthreads) */
	uint8_t* sW = tsm;
	uint8_t* sA = tsm + kTcWBytes + (size_t) g * kTcABytes;
	float* sB = (float*) (tsm + kTcWBytes + (size_t) kLearnGroups * kTcABytes);
	uint64_t* mbars = (uint64_t*) (sB + 208);
	uint32_t* tslot = (uint32_t*) (mbars + kLearnGroups);
	uint32_t* sNext = tslot + 4;                       /* per group: the pair it takes next */
	for (int i = tid; i < (int) (kTcWBytes / 16); i += kLearnThreads) ((uint4*) sW)[i] = ((const uint4*) P.mlpW5)[i];
	for (int i = tid; i < 3 * kMlpHid + kMlpOut; i += kLearnThreads) sB[i] = P.mlpB[i];
	const uint32_t mb = smemAddr(mbars + g);
	if (gt == 0) {
		mbarInit(mb, 1);
		sNext[g] = atomicAdd(&P.ctr->learnedPairs, 1u);
	}
	if (warp == 0) tcAlloc(smemAddr(tslot), kLearnCols);
	fenceProxyAsync();
	tcFenceBefore();
	__syncthreads();
	tcFenceAfter();
	const uint32_t tmemAll = *tslot;
	const uint32_t tmem = tmemAll + (uint32_t) (g * 64);
	const uint32_t laneBase = tmem + ((uint32_t) ((warp & 3) * 32) << 16);
	const uint32_t aAddr = smemAddr(sA), wAddr = smemAddr(sW);
	const int half = gt >> 6, q = gt & 63;
	uint32_t phase = 0;
	bool ok = P.ctr->abort == 0;
	const uint32_t pairs = (numTiles + 1) / 2;
	for (uint32_t pr = sNext[g]; ok && pr < pairs; pr = sNext[g]) {
		/* sNext[g] is rewritten only after the group's next barrier, once every thread has read it */
		const uint32_t tile = 2 * pr + (uint32_t) half;
		const bool have = tile < numTiles && P.tileStart[tile] < P.tileEnd[tile];
		TileCtx c = {};
		size_t idx = 0;
		int32_t win = -1;
		float x9[9] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
		if (have) {
			c = tileCtx<MULTI>(P, tile);
			const int gx = c.x0 + (q & 7), gy = c.y0 + (q >> 3);
			if (gx < c.W && gy < c.H) {
				idx = (size_t) gy * c.W + gx;
				win = c.winner[idx];
			}
			if (win >= 0) {
				uint32_t words[kMaxVaryingWords];
				SRPFragmentShaderIn in;
				fragmentIn<KIND>(P, c.uniform, c.primBase, (uint32_t) win, gx, gy, in, words);
				learnedInputs(c.uniform, words, x9);
			}
		}
		const bool any = namedSyncOr(bar, 128, win >= 0);
		uint32_t next = 0;
		if (gt == 0) next = atomicAdd(&P.ctr->learnedPairs, 1u);
		if (!any) {
			if (gt == 0) sNext[g] = next;
			namedSync(bar, 128);
			continue;
		}
#pragma unroll
		for (int f = 0; f < kMlpInPad; f += 2) {
			uint32_t v = 0;
			if (f < kMlpIn) {
				float sn, cs;
				__sincosf(mlpBandScale((f % 12) / 2) * x9[f / 12], &sn, &cs);
				v = packBf16(sn, cs);
			}
			*(uint32_t*) (sA + tcOffset(gt, f, kMlpInPad)) = v;
		}
		fenceProxyAsync();
		tcFenceBefore();
		namedSync(bar, 128);
		float rgb[3] = { 0.f, 0.f, 0.f };
		for (int layer = 0; layer < 4; ++layer) {
			/* a failure-detection test issues nothing for layer 1: its wait
			 * runs out with no MMA in flight */
			if (gt == 0 && !(layer == 1 && (P.waitTest & kWaitTestLearned))) {
				tcFenceAfter();
				const int K = layer == 0 ? kMlpInPad : 64;
				const uint32_t w = wAddr + (layer == 0 ? kTcW1 : layer == 1 ? kTcW2 : layer == 2 ? kTcW3 : kTcW4);
				tcLayer(tmem, aAddr, w, K, layer < 3 ? 64 : 16);
				tcCommit(mb);
				/* the counter's answer is awaited here, beside the first layer's MMAs */
				if (layer == 0) sNext[g] = next;
			}
			const bool got = mbarWait(mb, phase, P.spinLimit);
			phase ^= 1u;
			if (!namedSyncAnd(bar, 128, got)) { ok = false; break; }
			tcFenceAfter();
			if (layer < 3) {
				const float* bias = sB + 64 * layer;
				for (int col = 0; col < 64; col += 16) {
					float v[16];
					tcLoad16(laneBase + (uint32_t) col, v);
#pragma unroll
					for (int i = 0; i < 16; i += 2) {
						const float x0 = fmaxf(v[i] + bias[col + i], 0.0f), x1 = fmaxf(v[i + 1] + bias[col + i + 1], 0.0f);
						*(uint32_t*) (sA + tcOffset(gt, col + i, 64)) = packBf16(x0, x1);
					}
				}
				fenceProxyAsync();
			} else {
				float v[16];
				tcLoad16(laneBase, v);
				for (int k = 0; k < 3; ++k) rgb[k] = clamp01f(v[k] + sB[3 * kMlpHid + k]);
			}
			tcFenceBefore();
			namedSync(bar, 128);
		}
		if (!ok) break;
		if (win >= 0) {
			const float col[4] = { rgb[0], rgb[1], rgb[2], 1.0f };
			c.color[idx] = packColor(col);
		}
	}
	if (!ok && P.ctr->abort == 0 && gt == 0) atomicOr(&P.ctr->errors, kErrSpin);
	tcFenceBefore();
	__syncthreads();
	tcFenceAfter();
	if (warp == 0) tcDealloc(tmemAll, kLearnCols);
}

/* The judge of learned shading, a pass of its own after k_shade_learned5:
 * 1 pixel in judgeEvery is shaded again by the plain shader (FS), and per
 * draw the squared difference between the network's stored colour and the
 * shader's (both as the 8-bit channels the framebuffer holds, in [0, 1]
 * units) and the largest channel difference are accumulated. Run at the
 * deferred-shading pass's occupancy, so that the few judged pixels do not
 * hold up the tensor-core kernel's tile pairs. */
template <int KIND, int FS, bool MULTI>
__global__ void __launch_bounds__(kShadeTiles * 64) k_judge_learned(const __grid_constant__ DrawParams P, uint32_t numTiles)
{
	gridDepSync();
	const uint32_t tile = blockIdx.x * kShadeTiles + (threadIdx.x >> 6);
	const int q = threadIdx.x & 63;
	/* tile-level exits are uniform over each warp: a warp's 32 pixels lie in one tile */
	if (tile >= numTiles || P.ctr->abort) return;
	if (P.tileStart[tile] >= P.tileEnd[tile]) return;
	const TileCtx c = tileCtx<MULTI>(P, tile);
	const int gx = c.x0 + (q & 7), gy = c.y0 + (q >> 3);
	double err = 0.0, chans = 0.0;
	float worst = 0.0f;
	if (gx < c.W && gy < c.H && pixelSampled(gx, gy, P.sampleSeed + c.d, P.judgeEvery)) {
		const size_t idx = (size_t) gy * c.W + gx;
		const int32_t w = c.winner[idx];
		if (w >= 0) {
			SRPFragmentShaderOut ref;
			shadeItem<KIND, FS>(P, c.uniform, c.primBase, (uint32_t) w, gx, gy, ref);
			const uint32_t net = c.color[idx], plain = packColor(ref.color);
			for (int k = 0; k < 3; ++k) {
				const int sh = 24 - 8 * k;
				const float dlt = (float) ((int) ((net >> sh) & 0xFFu) - (int) ((plain >> sh) & 0xFFu)) / 255.0f;
				err += (double) dlt * dlt;
				worst = fmaxf(worst, fabsf(dlt));
			}
			chans = 3.0;
		}
	}
	for (int o = 16; o; o >>= 1) {
		err += __shfl_xor_sync(0xFFFFFFFFu, err, o);
		chans += __shfl_xor_sync(0xFFFFFFFFu, chans, o);
		worst = fmaxf(worst, __shfl_xor_sync(0xFFFFFFFFu, worst, o));
	}
	if ((threadIdx.x & 31) == 0 && chans > 0.0) {
		atomicAdd(&P.judge[2 * c.d], err);
		atomicAdd(&P.judge[2 * c.d + 1], chans);
		atomicMax(&P.judgeMax[c.d], __float_as_uint(worst));
	}
}

/* ------------------------------------------------------------ launchers */

static unsigned tileBlocks(uint32_t numTiles) { return (numTiles + kResolveWarps - 1) / kResolveWarps; }

template <int KIND, bool MULTI = false>
static void launchHeavy(const DrawParams& P, const uint32_t* vals, uint32_t* heavy, cudaStream_t s)
{
	const int smem = kHeavyThreads * kDepRow * 4;
	cudaFuncSetAttribute(k_resolve_heavy<KIND, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
	const unsigned perSM = P.heavyCtasPerSM >= 1 && P.heavyCtasPerSM <= 3 ? P.heavyCtasPerSM : 3u;
	pdlLaunch(k_resolve_heavy<KIND, MULTI>, 152 * perSM, kHeavyThreads, smem, s, P, vals, heavy);
}

void launchResolve(const DrawParams& P, int kind, const uint32_t* vals, uint32_t numTiles, uint32_t* heavy, cudaStream_t s,
                   cudaStream_t aux, cudaEvent_t fork, cudaEvent_t join)
{
	const unsigned b = tileBlocks(numTiles);
	pdlLaunch(k_tile_classify, (numTiles + 255) / 256, 256, 0, s, P, numTiles, heavy);
	const bool split = aux && fork && join;
	cudaStream_t hs = s;
	if (split) {
		cudaEventRecord(fork, s);
		cudaStreamWaitEvent(aux, fork, 0);
		hs = aux;
	}
	if (kind == kKindTri) {
		launchHeavy<kKindTri>(P, vals, heavy, hs);
		pdlLaunch(k_resolve<kKindTri, 0>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	} else if (kind == kKindPoint) {
		launchHeavy<kKindPoint>(P, vals, heavy, hs);
		pdlLaunch(k_resolve<kKindPoint, 0>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	} else {
		launchHeavy<kKindLineFrag>(P, vals, heavy, hs);
		pdlLaunch(k_resolve_frags, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	}
	if (split) {
		cudaEventRecord(join, aux);
		cudaStreamWaitEvent(s, join, 0);
	}
}

bool shadeSupportsLateDepth(int fsId) { return fsId == SRP_GPU_FS_DEPTH_OVERWRITE; }

void launchResolveLate(const DrawParams& P, int kind, const uint32_t* vals, uint32_t numTiles, cudaStream_t s)
{
	const unsigned b = tileBlocks(numTiles);
	if (kind == kKindTri) pdlLaunch(k_resolve<kKindTri, SRP_GPU_FS_DEPTH_OVERWRITE>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	else if (kind == kKindPoint) pdlLaunch(k_resolve<kKindPoint, SRP_GPU_FS_DEPTH_OVERWRITE>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	else pdlLaunch(k_resolve<kKindLineFrag, SRP_GPU_FS_DEPTH_OVERWRITE>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
}

template <int KIND, bool MULTI = false>
static void shadeKind(const DrawParams& P, uint32_t numTiles, cudaStream_t s)
{
	const unsigned b = (numTiles + kShadeTiles - 1) / kShadeTiles;
	const unsigned t = kShadeTiles * 64;
	switch (P.fsId) {
	case SRP_GPU_FS_VARYING_COLOR: pdlLaunch(k_shade<KIND, SRP_GPU_FS_VARYING_COLOR, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_SOLID: pdlLaunch(k_shade<KIND, SRP_GPU_FS_SOLID, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_PRIMITIVE_ID: pdlLaunch(k_shade<KIND, SRP_GPU_FS_PRIMITIVE_ID, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_TEXTURE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_TEXTURE, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_TEXTURE_MODULATE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_TEXTURE_MODULATE, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_BLINN_PHONG: pdlLaunch(k_shade<KIND, SRP_GPU_FS_BLINN_PHONG, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_MARBLE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_MARBLE, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_DEPTH_OVERWRITE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_DEPTH_OVERWRITE, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_FRAGCOORD: pdlLaunch(k_shade<KIND, SRP_GPU_FS_FRAGCOORD, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_FLAT_INT: pdlLaunch(k_shade<KIND, SRP_GPU_FS_FLAT_INT, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_MIXED: pdlLaunch(k_shade<KIND, SRP_GPU_FS_MIXED, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_BYTE_PALETTE: pdlLaunch(k_shade<KIND, SRP_GPU_FS_BYTE_PALETTE, MULTI>, b, t, 0, s, P, numTiles); break;
	case SRP_GPU_FS_PRIMITIVE_MOD: pdlLaunch(k_shade<KIND, SRP_GPU_FS_PRIMITIVE_MOD, MULTI>, b, t, 0, s, P, numTiles); break;
	case kFsLearned:
		if constexpr (KIND == kKindTri) {
			/* one CTA per SM, its groups looping over the tile pairs */
			const unsigned pairs = (numTiles + 1) / 2;
			const unsigned need = (pairs + kLearnGroups - 1) / kLearnGroups;
			const unsigned blocks = need < 152u ? (need ? need : 1u) : 152u;
			cudaFuncSetAttribute(k_shade_learned5<KIND, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kLearnSmem);
			pdlLaunch(k_shade_learned5<KIND, MULTI>, blocks, kLearnThreads, kLearnSmem, s, P, numTiles);
			pdlLaunch(k_judge_learned<KIND, SRP_GPU_FS_MARBLE, MULTI>, b, t, 0, s, P, numTiles);
		}
		break;
	default: break;
	}
}

void launchShade(const DrawParams& P, int kind, uint32_t numTiles, cudaStream_t s)
{
	if (kind == kKindTri) shadeKind<kKindTri>(P, numTiles, s);
	else if (kind == kKindPoint) shadeKind<kKindPoint>(P, numTiles, s);
	else shadeKind<kKindLineFrag>(P, numTiles, s);
}

void launchResolveMulti(const DrawParams& P, const uint32_t* vals, uint32_t numTiles, uint32_t* heavy, cudaStream_t s,
                        cudaStream_t aux, cudaEvent_t fork, cudaEvent_t join)
{
	const unsigned b = tileBlocks(numTiles);
	pdlLaunch(k_tile_classify, (numTiles + 255) / 256, 256, 0, s, P, numTiles, heavy);
	const bool split = aux && fork && join;
	cudaStream_t hs = s;
	if (split) {
		cudaEventRecord(fork, s);
		cudaStreamWaitEvent(aux, fork, 0);
		hs = aux;
	}
	launchHeavy<kKindTri, true>(P, vals, heavy, hs);
	pdlLaunch(k_resolve<kKindTri, 0, true>, b, kResolveWarps * 32, 0, s, P, vals, numTiles);
	if (split) {
		cudaEventRecord(join, aux);
		cudaStreamWaitEvent(s, join, 0);
	}
}

void launchShadeMulti(const DrawParams& P, uint32_t numTiles, cudaStream_t s) { shadeKind<kKindTri, true>(P, numTiles, s); }

}  // namespace srpg
