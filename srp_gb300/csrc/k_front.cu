/* Front end of a draw: vertex range, vertex shading, primitive assembly with
 * clipping and setup, ordered compaction, tile-pair emission, line DDA.
 *
 * Reference behaviour restated here (kitrofimov/srp):
 *   topology            src/pipeline/topology.c:14-83
 *   post-VS cache       src/pipeline/vertex_processing.c:23-74, 90-112
 *   clipping            src/pipeline/clipping.c:68-277
 *   triangle setup      src/raster/triangle.c:113-238
 *   line setup / DDA    src/raster/line.c:34-96
 *   point setup         src/raster/point.c:32-118
 *   numbering           src/pipeline/primitive_assembly.c:37-254
 * The reference numbers surviving primitives serially (post-clip, post-cull,
 * in submission order). Here one thread handles one input primitive; block
 * scans plus a decoupled look-back across blocks give every survivor the
 * same number, and the offset of its (tile, primitive) pairs, in one pass. */
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "kernels.h"
#include "launch.cuh"
#include "srp/buffer.h"

namespace srpg {
__device__ __forceinline__ void devTexSample(const void* tex, float u, float v, float out[4])
{
	textureSample((const TextureDesc*) tex, u, v, out);
}
__device__ __forceinline__ void devTexSampleLod(const void* tex, float u, float v, float lod, float out[4])
{
	textureSampleLod((const TextureDesc*) tex, u, v, lod, out);
}
}  // namespace srpg
#define SRP_DEVICE_TEXTURE_SAMPLE(tex, u, v, out) srpg::devTexSample((const void*) (tex), u, v, out)
#define SRP_DEVICE_TEXTURE_SAMPLE_LOD(tex, u, v, lod, out) srpg::devTexSampleLod((const void*) (tex), u, v, lod, out)
#include "srp/shaderlib_impl.h"

namespace srpg {

/* ----------------------------------------------------------- reset/range */

__global__ void k_reset(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (threadIdx.x == 0) {
		/* per-draw counters start at zero; the fragment total accumulates */
		DeviceCounters c = {};
		c.fragments = P.ctr->fragments;
		*P.ctr = c;
		P.minmax[0] = ~0ull;
		P.minmax[1] = 0ull;
	}
}

/* Abort flag of a draw (one thread, after setup): any count above the
 * buffer it was meant for, or a bad index, stops the rest of the draw. */
__global__ void k_check(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (threadIdx.x != 0) return;
	const DeviceCounters& c = *P.ctr;
	const bool over = c.clipVerts > P.clipCap || c.prims > P.primCap || c.entries > P.entryCap ||
	                  c.bigJobs > P.bigCap || c.tableWords > P.tableCap || c.clipTris > P.clipPolyCap;
	if (over || (c.errors & (kErrCapacity | kErrBadIndex | kErrSpin))) P.ctr->abort = 1u;
}

__device__ __forceinline__ unsigned long long fetchIndexRaw(const void* indices, int indexSize, unsigned long long i)
{
	switch (indexSize) {
	case 1: return ((const uint8_t*) indices)[i];
	case 2: return ((const uint16_t*) indices)[i];
	case 4: return ((const uint32_t*) indices)[i];
	case 8: return ((const unsigned long long*) indices)[i];
	default: return i;
	}
}

__device__ __forceinline__ unsigned long long fetchIndex(const DrawParams& P, unsigned long long i)
{
	return fetchIndexRaw(P.indices, P.indexSize, i);
}

/* Min/max over the elements of one aligned 16-byte word of the index
 * buffer: all of them when the word lies inside the draw's byte range
 * [b0, b1), else only those inside it. */
template <typename I>
__device__ __forceinline__ void wordRange(const uint4& q, unsigned long long at, unsigned long long b0,
                                          unsigned long long b1, unsigned long long& lo, unsigned long long& hi)
{
	constexpr int n = 16 / (int) sizeof(I);
	I e[n];
	memcpy(e, &q, 16);
	const bool whole = at >= b0 && at + 16 <= b1;
#pragma unroll
	for (int k = 0; k < n; ++k) {
		const unsigned long long off = at + (unsigned long long) k * sizeof(I);
		if (whole || (off >= b0 && off < b1)) {
			const unsigned long long v = (unsigned long long) e[k];
			lo = v < lo ? v : lo;
			hi = v > hi ? v : hi;
		}
	}
}

/* min/max vertex index over the draw's index range
 * (src/pipeline/vertex_processing.c:90-112). The range's bytes are read as
 * aligned 16-byte words, two independent loads per thread per iteration, so
 * that enough bytes are in flight to stream the index buffer at HBM speed.
 * Boundary words can reach up to 15 bytes past the last index: index
 * buffers are allocated with 16 bytes of slack. */
__global__ void k_index_range(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	const unsigned long long isz = (unsigned long long) P.indexSize;
	const unsigned long long b0 = P.start * isz, b1 = (P.start + P.count) * isz;
	const unsigned long long w0 = b0 >> 4, w1 = (b1 + 15) >> 4;
	const uint4* words = (const uint4*) P.indices;
	const unsigned long long stride = (unsigned long long) gridDim.x * blockDim.x;
	unsigned long long lo = ~0ull, hi = 0;
	for (unsigned long long w = w0 + blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; w < w1; w += 2 * stride) {
		const bool two = w + stride < w1;
		const uint4 a = __ldg(words + w);
		const uint4 b = two ? __ldg(words + w + stride) : a;
		switch (isz) {
		case 1: wordRange<uint8_t>(a, w << 4, b0, b1, lo, hi); wordRange<uint8_t>(b, (two ? w + stride : w) << 4, b0, b1, lo, hi); break;
		case 2: wordRange<uint16_t>(a, w << 4, b0, b1, lo, hi); wordRange<uint16_t>(b, (two ? w + stride : w) << 4, b0, b1, lo, hi); break;
		case 4: wordRange<uint32_t>(a, w << 4, b0, b1, lo, hi); wordRange<uint32_t>(b, (two ? w + stride : w) << 4, b0, b1, lo, hi); break;
		default: wordRange<unsigned long long>(a, w << 4, b0, b1, lo, hi); wordRange<unsigned long long>(b, (two ? w + stride : w) << 4, b0, b1, lo, hi); break;
		}
	}
	/* warp, then block reduction: two atomics per block on the shared pair */
	__shared__ unsigned long long sLo[8], sHi[8];
	for (int o = 16; o; o >>= 1) {
		const unsigned long long l2 = __shfl_xor_sync(0xFFFFFFFFu, lo, o);
		const unsigned long long h2 = __shfl_xor_sync(0xFFFFFFFFu, hi, o);
		lo = l2 < lo ? l2 : lo;
		hi = h2 > hi ? h2 : hi;
	}
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	if (lane == 0) { sLo[warp] = lo; sHi[warp] = hi; }
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int w = 1; w < (int) (blockDim.x >> 5); ++w) {
			lo = sLo[w] < lo ? sLo[w] : lo;
			hi = sHi[w] > hi ? sHi[w] : hi;
		}
		if (lo != ~0ull) atomicMin(&P.minmax[0], lo);
		if (hi != 0ull) atomicMax(&P.minmax[1], hi);
	}
}

/* ------------------------------------------------- per-vertex setup data */

struct PV { float4 p; uint32_t ref; };

/* Per-vertex results of the reference's perspective divide and viewport
 * transform (src/pipeline/vertex_processing.c:76-88,
 * src/core/framebuffer.c:48-55). The reference recomputes them for every
 * primitive corner from the same clip position, so they are a pure function
 * of the vertex and are computed once per vertex by k_vertex; clipping
 * creates new vertices, whose values are computed on the spot. */
struct VSet { float nx, ny, nz, sx, sy, c, iw; };
struct SV { VSet s; uint32_t ref; };

__device__ __forceinline__ VSet vertexSetup(int W, int H, const float4& clip)
{
	VSet v;
	v.iw = invW(clip.w);
	v.nx = __fmul_rn(clip.x, v.iw);
	v.ny = __fmul_rn(clip.y, v.iw);
	v.nz = __fmul_rn(clip.z, v.iw);
	ndcToScreen(W, H, v.nx, v.ny, v.sx, v.sy);
	v.c = __fmul_rn(v.nz, v.iw);
	return v;
}

__device__ __forceinline__ VSet vertexSetup(const DrawState& st, const float4& clip)
{
	return vertexSetup(st.W, st.H, clip);
}

__device__ __forceinline__ SV fromClip(int W, int H, const PV& p)
{
	SV v;
	v.s = vertexSetup(W, H, p.p);
	v.ref = p.ref;
	return v;
}

__device__ __forceinline__ SV fromClip(const DrawState& st, const PV& p)
{
	return fromClip(st.W, st.H, p);
}

enum SetupMode { kTriFill = 0, kTriLine = 1, kTriPoint = 2, kLines = 3, kPoints = 4 };

__device__ __forceinline__ float planeDist(const float4& c, int p)
{
	/* src/pipeline/clipping.c:260-277 */
	switch (p) {
	case 0: return __fadd_rn(c.x, c.w);
	case 1: return __fsub_rn(c.w, c.x);
	case 2: return __fadd_rn(c.y, c.w);
	case 3: return __fsub_rn(c.w, c.y);
	case 4: return __fadd_rn(c.z, c.w);
	default: return __fsub_rn(c.w, c.z);
	}
}

__device__ __forceinline__ uint32_t outcode(const float4& c)
{
	/* src/pipeline/clipping.c:121-137 */
	uint32_t code = 0;
#pragma unroll
	for (int p = 0; p < 6; ++p) code |= (uint32_t) (planeDist(c, p) < 0.0f) << p;
	return code;
}


/* --------------------------------------------------------------- vertex */

constexpr int kVertexThreads = 128;

template <int VS>
__device__ __forceinline__ void runVS(SRPVertexShaderIn* in, SRPVertexShaderOut* out)
{
	if (VS == SRP_GPU_VS_TRANSFORM) srpslVsTransform(in, out);
	else if (VS == SRP_GPU_VS_WORLD) srpslVsWorld(in, out);
	else if (VS == SRP_GPU_VS_BYTES) srpslVsBytes(in, out);
}

/* One thread per vertex of [lo, hi]: the block's vertex records (a
 * contiguous byte range of the user's AoS buffer) are staged through shared
 * memory with coalesced word loads, each thread runs the vertex shader on its
 * record, and writes the clip position and varying words. Running every
 * vertex of the referenced range exactly once gives the same outputs as the
 * reference's post-VS cache (the shader is a pure function of its inputs). */
template <int VS>
__global__ void __launch_bounds__(kVertexThreads) k_vertex(const __grid_constant__ DrawParams P,
                                                             unsigned long long first, unsigned long long n)
{
	gridDepSync();
	extern __shared__ uint32_t stage[];
	unsigned long long lo, hi;
	if (P.indexSize && P.shadeAll) { lo = 0; hi = P.nVertices ? P.nVertices - 1 : 0; }
	else if (P.indexSize) { lo = P.minmax[0]; hi = P.minmax[1]; }
	else { lo = P.start; hi = P.start + P.count - 1; }
	if (hi >= P.nVertices) {
		if (threadIdx.x == 0 && blockIdx.x == 0 && P.indexSize) atomicOr(&P.ctr->errors, kErrBadIndex);
		hi = P.nVertices ? P.nVertices - 1 : 0;
	}
	const unsigned long long vb = first + (unsigned long long) blockIdx.x * kVertexThreads;
	if (vb > hi || vb + kVertexThreads <= lo || P.nVertices == 0) return;
	const unsigned long long vend = (vb + kVertexThreads < first + n) ? vb + kVertexThreads : first + n;
	const int stride = P.stride;
	const unsigned long long bytes = (vend - vb) * (unsigned long long) stride;
	const unsigned char* src = P.vertices + vb * (unsigned long long) stride;
	if ((stride & 3) == 0) {
		const uint32_t* w = (const uint32_t*) src;
		for (unsigned long long i = threadIdx.x; i < bytes / 4; i += kVertexThreads) stage[i] = __ldg(w + i);
	} else {
		unsigned char* sb = (unsigned char*) stage;
		for (unsigned long long i = threadIdx.x; i < bytes; i += kVertexThreads) sb[i] = __ldg(src + i);
	}
	__syncthreads();
	const unsigned long long v = vb + threadIdx.x;
	if (v >= vend || v < lo || v > hi) return;
	uint32_t vtx[kMaxVertexWords];
	const unsigned char* rec = (const unsigned char*) stage + (unsigned long long) threadIdx.x * stride;
	const int words = (stride + 3) / 4 < kMaxVertexWords ? (stride + 3) / 4 : kMaxVertexWords;
#pragma unroll
	for (int k = 0; k < kMaxVertexWords; ++k) vtx[k] = 0;
	if ((stride & 3) == 0) {
#pragma unroll
		for (int k = 0; k < kMaxVertexWords; ++k)
			if (k < words) vtx[k] = ((const uint32_t*) rec)[k];
	} else {
		memcpy(vtx, rec, stride < 4 * kMaxVertexWords ? stride : 4 * kMaxVertexWords);
	}
	uint32_t out[kMaxVaryingWords];
#pragma unroll
	for (int k = 0; k < kMaxVaryingWords; ++k) out[k] = 0;
	SRPVertexShaderIn in;
	in.uniform = (SRPUniform*) P.uniform;
	in.vertex = (SRPVertex*) vtx;
	in.vertexID = (size_t) v;
	SRPVertexShaderOut o;
	o.clipPosition[0] = o.clipPosition[1] = o.clipPosition[2] = o.clipPosition[3] = 0.0f;
	o.varyings = (SRPVarying*) out;
	runVS<VS>(&in, &o);
	const float4 clip = make_float4(o.clipPosition[0], o.clipPosition[1], o.clipPosition[2], o.clipPosition[3]);
	P.clip[v] = clip;
	/* setup data is read only for vertices inside the frustum (outcode 0):
	 * every primitive with an outside vertex is rejected or re-derived from
	 * clip coordinates, so the divide and the double-precision viewport step
	 * are skipped for outside vertices */
	const uint32_t code = outcode(clip);
	P.codes[v] = (uint8_t) code;
	if (code == 0) {
		const VSet vs = vertexSetup(P.st, clip);
		P.vset0[v] = make_float4(vs.nx, vs.ny, vs.sx, vs.sy);
		P.vset1[v] = make_float4(vs.c, vs.iw, vs.nz, __uint_as_float(0u));
	}
	const int nw = P.L.nWords;
	uint32_t* dst = P.vary + v * (unsigned long long) nw;
#pragma unroll
	for (int k = 0; k < kMaxVaryingWords; ++k)
		if (k < nw) dst[k] = out[k];
}

/* ----------------------------------------------------------------- setup */

/* New vertex a*(1-t) + b*t with affinely interpolated varyings, stored as a
 * clip-generated row (src/pipeline/clipping.c:244-258). */
__device__ PV lerpVertex(const DrawParams& P, const PV& a, const PV& b, float t)
{
	PV o;
	const float s = __fsub_rn(1.0f, t);
	o.p.x = __fadd_rn(__fmul_rn(a.p.x, s), __fmul_rn(b.p.x, t));
	o.p.y = __fadd_rn(__fmul_rn(a.p.y, s), __fmul_rn(b.p.y, t));
	o.p.z = __fadd_rn(__fmul_rn(a.p.z, s), __fmul_rn(b.p.z, t));
	o.p.w = __fadd_rn(__fmul_rn(a.p.w, s), __fmul_rn(b.p.w, t));
	const unsigned long long slot = atomicAdd(&P.ctr->clipVerts, 1ull);
	if (slot >= P.clipCap) {
		atomicOr(&P.ctr->errors, kErrCapacity);
		o.ref = a.ref;
		return o;
	}
	o.ref = P.clipBase + (uint32_t) slot;
	const uint32_t refs[2] = { a.ref, b.ref };
	const float w[2] = { s, t };
	const float iw[2] = { 1.0f, 1.0f };
	uint32_t words[kMaxVaryingWords];
	interpolate<2>(P.L, P.vary, refs, w, iw, 0.0f, P.st.provokingFirst, true, words);
	const int nw = P.L.nWords;
	P.clip[o.ref] = o.p;
	for (int k = 0; k < nw; ++k) P.vary[(size_t) o.ref * nw + k] = words[k];
	return o;
}

/* Sutherland-Hodgman against L, R, B, T, N, F (src/pipeline/clipping.c:68-119,
 * 199-242). Returns the polygon size; out has room for kMaxPoly vertices. */
__device__ __noinline__ int clipPolygon(const DrawParams& P, const PV in[3], PV out[kMaxPoly])
{
	PV a[kMaxPoly], b[kMaxPoly];
	int n = 3;
	for (int i = 0; i < 3; ++i) a[i] = in[i];
	PV* src = a;
	PV* dst = b;
	for (int p = 0; p < 6; ++p) {
		int m = 0;
		for (int i = 0; i < n; ++i) {
			const PV& cur = src[i];
			const PV& nxt = src[(i + 1) % n];
			const float da = planeDist(cur.p, p), db = planeDist(nxt.p, p);
			const bool cin = da >= 0.0f, nin = db >= 0.0f;
			if (cin && nin) {
				if (m < kMaxPoly) dst[m++] = nxt;
			} else if (cin || nin) {
				const float diff = __fsub_rn(da, db);
				if (roughlyZero(diff)) continue;
				const float t = __fdiv_rn(da, diff);
				if (m < kMaxPoly) dst[m++] = lerpVertex(P, cur, nxt, t);
				if (!cin && nin && m < kMaxPoly) dst[m++] = nxt;
			}
		}
		n = m;
		if (n == 0) return 0;
		PV* tmp = src; src = dst; dst = tmp;
	}
	if (n > 6) atomicAdd(&P.ctr->clipOverflow, 1ull);
	for (int i = 0; i < n; ++i) out[i] = src[i];
	return n;
}

/* Liang-Barsky (src/pipeline/clipping.c:139-183); returns true if rejected. */
__device__ bool clipLine(const DrawParams& P, PV& v0, PV& v1)
{
	const uint32_t c0 = outcode(v0.p), c1 = outcode(v1.p);
	if ((c0 | c1) == 0) return false;
	if (c0 & c1) return true;
	float t0 = 0.0f, t1 = 1.0f;
	for (int p = 0; p < 6; ++p) {
		const float da = planeDist(v0.p, p), db = planeDist(v1.p, p);
		if (da < 0.0f && db < 0.0f) return true;
		if (da < 0.0f || db < 0.0f) {
			const float diff = __fsub_rn(da, db);
			if (roughlyZero(diff)) continue;
			const float t = __fdiv_rn(da, diff);
			if (da < 0.0f) t0 = t0 > t ? t0 : t;
			else t1 = t1 > t ? t : t1;
			if (t0 > t1) return true;
		}
	}
	const PV a = v0, b = v1;
	if (t0 > 0.0f) v0 = lerpVertex(P, a, b, t0);
	if (t1 < 1.0f) v1 = lerpVertex(P, a, b, t1);
	return false;
}

__device__ __forceinline__ uint32_t tileCount(int minX, int minY, int maxXex, int maxYex)
{
	if (maxXex <= minX || maxYex <= minY) return 0;
	return (uint32_t) ((maxXex - 1) / kTile - minX / kTile + 1) * (uint32_t) ((maxYex - 1) / kTile - minY / kTile + 1);
}

/* The inclusive pixel box [x0, x1] x [y0, y1] (x0, y0 >= 0) cut to the
 * scissor rectangle: a pixel outside it fails the scissor test before any
 * other test or write (src/raster/fragment.c:63-75), so tiles outside it need
 * no (tile, item) pair. Returns false when nothing is left. */
__device__ __forceinline__ bool scissorBox(const DrawState& st, int& x0, int& y0, int& x1, int& y1)
{
	if (x1 < x0 || y1 < y0) return false;
	if (!st.scissorEnabled) return true;
	if (st.sx1 <= st.sx0 || st.sy1 <= st.sy0) return false;
	const uint64_t lx = max((uint64_t) x0, st.sx0), hx = min((uint64_t) x1, st.sx1 - 1);
	const uint64_t ly = max((uint64_t) y0, st.sy0), hy = min((uint64_t) y1, st.sy1 - 1);
	if (lx > hx || ly > hy) return false;
	x0 = (int) lx; x1 = (int) hx; y0 = (int) ly; y1 = (int) hy;
	return true;
}

/* Bounding boxes of at most this many pixels a side are tested pixel by
 * pixel at setup. */
constexpr int kTinyTri = 3;

/* A triangle's bounding box cut to the scissor rectangle. */
__device__ __forceinline__ bool triScissorBox(const DrawState& st, const TriRaster& R, int& x0, int& y0, int& x1, int& y1)
{
	x0 = R.minX; y0 = R.minY; x1 = (int) R.maxX - 1; y1 = (int) R.maxY - 1;
	return scissorBox(st, x0, y0, x1, y1);
}

/* Whether a pixel centre of [x0, x1] x [y0, y1] (inside the bounding box)
 * passes the inside test, walking the box from its first pixel as the
 * reference does (src/raster/triangle.c:73-111): the same serial fp32 adds
 * the resolve's exact chain reproduces, so the answer is the resolve's. */
__device__ __forceinline__ bool triCoversBox(const TriRaster& R, int x0, int y0, int x1, int y1)
{
	float row[3] = { R.l0[0], R.l0[1], R.l0[2] };
	for (int y = (int) R.minY; y <= y1; ++y) {
		if (y >= y0) {
			float l[3] = { row[0], row[1], row[2] };
			for (int x = (int) R.minX; x <= x1; ++x) {
				if (x >= x0 && insideTri(l, R.flags)) return true;
#pragma unroll
				for (int i = 0; i < 3; ++i) l[i] = __fadd_rn(l[i], R.dx[i]);
			}
		}
#pragma unroll
		for (int i = 0; i < 3; ++i) row[i] = __fadd_rn(row[i], R.dy[i]);
	}
	return false;
}

/* Tiles that get a (tile, triangle) pair: those of the bounding box cut to the
 * scissor, or none when the triangle covers no pixel centre there. Most
 * triangles of a dense mesh seen from afar are smaller than a pixel; for a
 * bounding box of at most kTinyTri x kTinyTri pixels every pixel centre is
 * tested, so a triangle is dropped only when the resolve would find no
 * fragment in it either. It keeps its primitive number. Writers emit over
 * triScissorBox when this count is not zero. */
__device__ __forceinline__ uint32_t triPairTiles(const DrawState& st, const TriRaster& R)
{
	int x0, y0, x1, y1;
	if (!triScissorBox(st, R, x0, y0, x1, y1)) return 0u;
	if ((int) R.maxX - (int) R.minX <= kTinyTri && (int) R.maxY - (int) R.minY <= kTinyTri &&
	    !triCoversBox(R, x0, y0, x1, y1))
		return 0u;
	return tileCount(x0, y0, x1 + 1, y1 + 1);
}

/* Pixel box of a point's pairs: its raster bounds cut to the scissor. */
__device__ __forceinline__ bool pointPairBox(const DrawState& st, const PointRec& R, int& x0, int& y0, int& x1, int& y1)
{
	x0 = R.x0; y0 = R.y0; x1 = R.x1; y1 = R.y1;
	return scissorBox(st, x0, y0, x1, y1);
}

__device__ __forceinline__ uint32_t pointPairTiles(const DrawState& st, const PointRec& R)
{
	int x0, y0, x1, y1;
	return pointPairBox(st, R, x0, y0, x1, y1) ? tileCount(x0, y0, x1 + 1, y1 + 1) : 0u;
}

/* Triangle setup (src/raster/triangle.c:113-238). Returns false if the
 * triangle is culled or degenerate. */
__device__ bool setupTriangle(const DrawState& st, int W, int H, const SV& v0, const SV& v1, const SV& v2, TriRaster& R,
                              TriAttr& A)
{
	float iw[3] = { v0.s.iw, v1.s.iw, v2.s.iw };
	float nx[3] = { v0.s.nx, v1.s.nx, v2.s.nx };
	float ny[3] = { v0.s.ny, v1.s.ny, v2.s.ny };
	float cz[3] = { v0.s.c, v1.s.c, v2.s.c };
	float sx[3] = { v0.s.sx, v1.s.sx, v2.s.sx };
	float sy[3] = { v0.s.sy, v1.s.sy, v2.s.sy };
	uint32_t ref[3] = { v0.ref, v1.ref, v2.ref };
	/* NDC cull (triangle.c:162-182) */
	const float e0x = __fsub_rn(nx[1], nx[0]), e0y = __fsub_rn(ny[1], ny[0]);
	const float e1x = __fsub_rn(nx[2], nx[0]), e1y = __fsub_rn(ny[2], ny[0]);
	const float area = __fsub_rn(__fmul_rn(e0x, e1y), __fmul_rn(e0y, e1x));
	const bool front = ((area > 0.0f) && !st.frontFaceCW) || ((area < 0.0f) && st.frontFaceCW);
	if ((front && st.cullFace == SRP_FACE_FRONT) || (!front && st.cullFace == SRP_FACE_BACK)) return false;
	if (!(area > 0.0f)) {
		/* winding fix: swap vertices 1 and 2 (triangle.c:184-195) */
		float t;
		t = iw[1]; iw[1] = iw[2]; iw[2] = t;
		t = cz[1]; cz[1] = cz[2]; cz[2] = t;
		t = sx[1]; sx[1] = sx[2]; sx[2] = t;
		t = sy[1]; sy[1] = sy[2]; sy[2] = t;
		uint32_t r = ref[1]; ref[1] = ref[2]; ref[2] = r;
	}
	float ex[3], ey[3];
#pragma unroll
	for (int i = 0; i < 3; ++i) {
		ex[i] = __fsub_rn(sx[(i + 1) % 3], sx[i]);
		ey[i] = __fsub_rn(sy[(i + 1) % 3], sy[i]);
	}
	const float areaX2 = fabsf(__fsub_rn(__fmul_rn(ex[0], ey[2]), __fmul_rn(ey[0], ex[2])));
	if (roughlyZero(areaX2)) return false;
	/* bbox with the reference's MIN/MAX macro semantics (triangle.c:142-149) */
	float m;
	m = sx[1] > sx[2] ? sx[2] : sx[1]; const float mnx = sx[0] > m ? m : sx[0];
	m = sy[1] > sy[2] ? sy[2] : sy[1]; const float mny = sy[0] > m ? m : sy[0];
	m = sx[1] > sx[2] ? sx[1] : sx[2]; const float mxx = sx[0] > m ? sx[0] : m;
	m = sy[1] > sy[2] ? sy[1] : sy[2]; const float mxy = sy[0] > m ? sy[0] : m;
	float fx = floorf(mnx), fy = floorf(mny), cx = ceilf(mxx), cy = ceilf(mxy);
	fx = fx > 0.0f ? fx : 0.0f;
	fy = fy > 0.0f ? fy : 0.0f;
	cx = cx > (float) W ? (float) W : cx;
	cy = cy > (float) H ? (float) H : cy;
	/* NaN coordinates compare false everywhere; the reference then walks an
	 * empty range, which clamping to an empty box reproduces. */
	if (!(fx <= (float) W)) fx = (float) W;
	if (!(fy <= (float) H)) fy = (float) H;
	if (!(cx >= 0.0f)) cx = 0.0f;
	if (!(cy >= 0.0f)) cy = 0.0f;
	R.minX = (uint16_t) fx; R.minY = (uint16_t) fy;
	R.maxX = (uint16_t) cx; R.maxY = (uint16_t) cy;
	/* barycentrics at the first pixel centre (triangle.c:197-226) */
	const float px = __fadd_rn(fx, 0.5f), py = __fadd_rn(fy, 0.5f);
	const float ax = __fsub_rn(px, sx[0]), ay = __fsub_rn(py, sy[0]);
	const float bx = __fsub_rn(px, sx[1]), by = __fsub_rn(py, sy[1]);
	const float qx = __fsub_rn(px, sx[2]), qy = __fsub_rn(py, sy[2]);
	R.l0[0] = __fdiv_rn(__fsub_rn(__fmul_rn(bx, ey[1]), __fmul_rn(by, ex[1])), areaX2);
	R.l0[1] = __fdiv_rn(__fsub_rn(__fmul_rn(qx, ey[2]), __fmul_rn(qy, ex[2])), areaX2);
	R.l0[2] = __fdiv_rn(__fsub_rn(__fmul_rn(ax, ey[0]), __fmul_rn(ay, ex[0])), areaX2);
	R.dx[0] = __fdiv_rn(ey[1], areaX2);
	R.dx[1] = __fdiv_rn(ey[2], areaX2);
	R.dx[2] = __fdiv_rn(ey[0], areaX2);
	R.dy[0] = __fdiv_rn(-ex[1], areaX2);
	R.dy[1] = __fdiv_rn(-ex[2], areaX2);
	R.dy[2] = __fdiv_rn(-ex[0], areaX2);
	uint32_t flags = front ? 1u : 0u;
#pragma unroll
	for (int i = 0; i < 3; ++i) {
		const bool tl = (ex[i] > 0.0f && roughlyZero(ey[i])) || (ey[i] < 0.0f);
		flags |= (tl ? 1u : 0u) << (1 + i);
		R.c[i] = cz[i];
		A.invW[i] = iw[i];
		A.vref[i] = ref[i];
	}
	R.flags = flags;
	R.table = kNoTable;
	A.pad = 0;
	return true;
}

/* Line setup: divide, screen space, DDA parameters
 * (src/raster/line.c:34-56, 79-86). */
__device__ void setupLine(const DrawState& st, const SV& a, const SV& b, LineRec& L)
{
	const float sx[2] = { a.s.sx, b.s.sx }, sy[2] = { a.s.sy, b.s.sy };
	L.invW[0] = a.s.iw; L.invW[1] = b.s.iw;
	L.c[0] = a.s.c; L.c[1] = b.s.c;
	const float dx = __fsub_rn(sx[1], sx[0]), dy = __fsub_rn(sy[1], sy[0]);
	float mx = fmaxf(fabsf(dx), fabsf(dy));
	int steps = (int) ceilf(mx);
	/* guard against non-finite or absurd coordinates (the reference would
	 * loop for billions of steps) */
	if (!(mx == mx) || mx > 1.0e6f) steps = 0;
	if (steps == 0) steps = 1;
	L.x0 = sx[0]; L.y0 = sy[0];
	L.xInc = __fdiv_rn(dx, (float) steps);
	L.yInc = __fdiv_rn(dy, (float) steps);
	L.tInc = __fdiv_rn(1.0f, (float) steps);
	L.steps = steps;
	L.vref[0] = a.ref; L.vref[1] = b.ref;
}

/* Line draws are binned as runs: a run is a maximal sequence of consecutive
 * DDA steps that pass the scissor test, land in the framebuffer and fall in
 * one tile. A line gets slots for its runs in the (tile, item) arrays; the
 * run in slot k keeps its fragments' records at k * kRunFrags + j, and its
 * pair carries k | count << kRunCountShift. */

constexpr uint32_t kShortLine = 48;   /* steps one thread walks on its own */

constexpr uint32_t kLineInside = 0x80000000u;

/* Tile distance (columns + rows) between two pixels with coordinates >= 0. */
__device__ __forceinline__ uint32_t tileDistance(int ax, int ay, int bx, int by)
{
	return (uint32_t) abs(ax / kTile - bx / kTile) + (uint32_t) abs(ay / kTile - by / kTile);
}

/* The far end of a coordinate's DDA: a value at least as far along the
 * line's direction as the accumulator after n steps. Each of the n fp32
 * additions rounds by at most half an ulp of the larger magnitude, i.e.
 * 2^-24 * max |value|, so the accumulated value lies within
 * n * 2^-24 * max |value| of the exact sum v0 + n * inc; twice that, plus a
 * little, bounds it. */
__device__ __forceinline__ int farPixel(float v0, float inc, uint32_t n)
{
	const double e = (double) v0 + (double) n * (double) inc;
	const double m = (double) n * fmax(fabs((double) v0), fabs(e)) * 0x1p-23 + 0x1p-10;
	const double f = inc >= 0.0f ? e + m : e - m;
	/* rounding half away from zero, as the walker rounds */
	return (int) fmax(fmin(round(f), 2.0e9), -2.0e9);
}

/* Pair slots for the runs of a line (L.slots, L.endPix), set after setupLine.
 * The DDA's pixel coordinates are monotone along the line. With its first
 * pixel and a pixel E at or beyond the one past its last step (farPixel) in
 * the framebuffer, every step lands in it; the steps that pass the scissor
 * rectangle are then consecutive (a monotone path through a rectangle), and
 * a walker visiting steps [a, b) finds at most tileDistance(pixel a,
 * pixel b) + 1 runs, E standing in for the pixel one past the end. A short
 * line has one walker; a long one has 32 (a warp's lanes, on consecutive
 * segments, the last one ending at E), whose bounds add up to
 * tileDistance(first pixel, E) + 32. Elsewhere a run may be a single step,
 * and the line gets a slot per step. */
__device__ __forceinline__ void lineRunInfo(const DrawState& st, LineRec& L)
{
	const uint32_t total = (uint32_t) L.steps + 1u;
	const int ax = (int) roundf(L.x0), ay = (int) roundf(L.y0);
	const int bx = farPixel(L.x0, L.xInc, total), by = farPixel(L.y0, L.yInc, total);
	const bool inside = ax >= 0 && ay >= 0 && bx >= 0 && by >= 0 && ax < st.W && bx < st.W && ay < st.H && by < st.H;
	uint32_t slots = total;
	if (inside) {
		const uint32_t walkers = total <= kShortLine ? 1u : 32u;
		const uint32_t d = tileDistance(ax, ay, bx, by) + walkers;
		if (d < slots) slots = d;
	}
	L.slots = slots | (inside ? kLineInside : 0u);
	L.endPix = ((uint32_t) bx & 0xFFFFu) | ((uint32_t) by << 16);
}

__device__ __forceinline__ uint32_t lineSlots(const LineRec& L) { return L.slots & ~kLineInside; }

/* Point setup: divide, screen space, coverage square and raster bounds
 * (src/raster/point.c:32-79, 121-163). */
__device__ void setupPoint(const DrawState& st, const SV& v, PointRec& R)
{
	const float sx = v.s.sx, sy = v.s.sy, nz = v.s.nz;
	const float half = __fmul_rn(st.pointSize, 0.5f);
	R.mnx = __fsub_rn(sx, half); R.mny = __fsub_rn(sy, half);
	R.mxx = __fadd_rn(sx, half); R.mxy = __fadd_rn(sy, half);
	R.z = nz;
	R.vref = v.ref;
	const float fx0 = floorf(R.mnx), fx1 = floorf(R.mxx), fy0 = floorf(R.mny), fy1 = floorf(R.mxy);
	/* the reference converts with (int); out-of-range values make the point
	 * fully off-screen there as well */
	int x0 = fx0 > -1.0e9f ? (fx0 < 1.0e9f ? (int) fx0 : 1000000000) : -1000000000;
	int x1 = fx1 > -1.0e9f ? (fx1 < 1.0e9f ? (int) fx1 : 1000000000) : -1000000000;
	int y0 = fy0 > -1.0e9f ? (fy0 < 1.0e9f ? (int) fy0 : 1000000000) : -1000000000;
	int y1 = fy1 > -1.0e9f ? (fy1 < 1.0e9f ? (int) fy1 : 1000000000) : -1000000000;
	if (x1 < 0 || y1 < 0 || x0 >= st.W || y0 >= st.H) { x0 = 1; x1 = 0; y0 = 1; y1 = 0; }
	else {
		if (x0 < 0) x0 = 0;
		if (y0 < 0) y0 = 0;
		if (x1 >= st.W) x1 = st.W - 1;
		if (y1 >= st.H) y1 = st.H - 1;
	}
	R.x0 = (int16_t) x0; R.x1 = (int16_t) x1; R.y0 = (int16_t) y0; R.y1 = (int16_t) y1;
}

/* Emit the (tile, item) pairs of an item whose pixels lie in the inclusive
 * pixel box [x0, x1] x [y0, y1]. Few tiles are written inline; the rest is
 * queued for k_big_entries. */
__device__ void emitEntries(const DrawParams& P, int kind, uint32_t item, uint32_t base, int x0, int y0, int x1, int y1)
{
	const uint32_t n = tileCount(x0, y0, x1 + 1, y1 + 1);
	if (n == 0) return;
	if (n <= (uint32_t) kSmallEntries) {
		uint32_t e = base;
		for (int ty = y0 / kTile; ty <= y1 / kTile; ++ty)
			for (int tx = x0 / kTile; tx <= x1 / kTile; ++tx, ++e)
				if (e < P.entryCap) { P.keys[e] = (uint32_t) (ty * P.st.tilesX + tx); P.vals[e] = item; }
		if (base + n > P.entryCap) atomicOr(&P.ctr->errors, kErrCapacity);
	} else {
		const unsigned long long j = atomicAdd(&P.ctr->bigJobs, 1ull);
		if (j < P.bigCap) P.bigJobs[j] = make_uint4(item, base, (uint32_t) kind, n);
		else atomicOr(&P.ctr->errors, kErrCapacity);
	}
}

/* Per-thread work on one input primitive: count (write == false) or write
 * the survivors at the given offsets. Clip-generated vertices are created in
 * the counting pass and kept in `poly` for the writing pass. */
template <int MODE>
struct Assembly {
	int nPoly;
	bool clipped;
	uint32_t slot;       /* clipped, filled: the pre-pass's slot of its fan */
	SV sv[3];            /* unclipped: per-vertex setup data from k_vertex */
	/* clipped triangles drawn as lines or points: polygon in clip space
	 * (filled triangles read their fan, set up by the pre-pass, instead) */
	PV poly[(MODE == kTriLine || MODE == kTriPoint) ? kMaxPoly : 1];
};

/* Write a set-up triangle as primitive `prim` with its pairs at `entry`. */
__device__ __forceinline__ void writeTri(const DrawParams& P, TriRaster& R, TriAttr& A, uint32_t nt, uint32_t prim,
                                         uint32_t entry)
{
			if (nt > (uint32_t) kSmallEntries) {
				/* big triangle: room for its lambda table */
				const int cols = ((int) R.maxX - 1) / kTile - (int) R.minX / kTile + 1;
				const unsigned long long words = 3ull * (unsigned long long) (R.maxY - R.minY) * (unsigned long long) cols;
				const unsigned long long off = atomicAdd(&P.ctr->tableWords, words);
				if (off + words <= P.tableCap && off < 0xFFFFFFFFull) R.table = (uint32_t) off;
			}
			if (prim < P.primCap) {
				A.id = prim;
				P.triR[prim] = R;
				P.triA[prim] = A;
				int x0, y0, x1, y1;
				if (nt && triScissorBox(P.st, R, x0, y0, x1, y1)) emitEntries(P, kKindTri, prim, entry, x0, y0, x1, y1);
			} else atomicOr(&P.ctr->errors, kErrCapacity);
}

template <int MODE>
__device__ __forceinline__ void handleTriangle(const DrawParams& P, const SV& a, const SV& b, const SV& c, bool write,
                                               uint32_t& prim, uint32_t& entry)
{
	if (MODE == kTriFill) {
		TriRaster R;
		TriAttr A;
		if (!setupTriangle(P.st, P.st.W, P.st.H, a, b, c, R, A)) return;
		const uint32_t nt = triPairTiles(P.st, R);
		if (write) writeTri(P, R, A, nt, prim, entry);
		prim += 1;
		entry += nt;
	} else if (MODE == kTriLine) {
		const SV* vv[3] = { &a, &b, &c };
#pragma unroll
		for (int j = 0; j < 3; ++j) {
			LineRec L;
			setupLine(P.st, *vv[j], *vv[(j + 1) % 3], L);
			lineRunInfo(P.st, L);
			if (write) {
				if (prim < P.primCap) { L.id = prim; L.fragBase = entry; P.lines[prim] = L; }
				else atomicOr(&P.ctr->errors, kErrCapacity);
			}
			prim += 1;
			entry += lineSlots(L);
		}
	} else if (MODE == kTriPoint) {
		const SV* vv[3] = { &a, &b, &c };
#pragma unroll
		for (int j = 0; j < 3; ++j) {
			PointRec R;
			setupPoint(P.st, *vv[j], R);
			const uint32_t nt = pointPairTiles(P.st, R);
			if (write) {
				if (prim < P.primCap) {
					R.id = prim;
					P.points[prim] = R;
					int x0, y0, x1, y1;
					if (pointPairBox(P.st, R, x0, y0, x1, y1)) emitEntries(P, kKindPoint, prim, entry, x0, y0, x1, y1);
				} else atomicOr(&P.ctr->errors, kErrCapacity);
			}
			prim += 1;
			entry += nt;
		}
	}
}

/* The fan of a clipped filled triangle (src/pipeline/clipping.c:139-183 then
 * triangle setup of each fan triangle, in fan order), set up by the clip
 * pre-pass into its slot: the triangles that survive setup, their records,
 * and their pair counts (tile pairs in a pass; the pair box otherwise).
 * The ordered setup then only copies them to their places. */
template <bool MULTI>
__device__ __noinline__ void setupClipFan(const DrawParams& P, uint32_t slot, const PV* poly, int n, int W, int H)
{
	uint32_t nP = 0, nE = 0;
	if (n >= 3) {
		const SV p0 = fromClip(W, H, poly[0]);
		for (int f = 1; f + 1 < n; ++f) {
			TriRaster R;
			TriAttr A;
			if (!setupTriangle(P.st, W, H, p0, fromClip(W, H, poly[f]), fromClip(W, H, poly[f + 1]), R, A)) continue;
			const uint32_t nt = MULTI ? tileCount(R.minX, R.minY, R.maxX, R.maxY) : triPairTiles(P.st, R);
			A.pad = nt;
			const size_t at = (size_t) slot * kClipFan + nP;
			P.clipR[at] = R;
			P.clipA[at] = A;
			nP += 1;
			nE += nt;
		}
	}
	P.clipFan[slot] = make_uint2(nP, nE);
}

/* Copies the fan of slot to primitives prim.. and pairs entry.. */
__device__ __forceinline__ void writeClipFan(const DrawParams& P, uint32_t slot, uint32_t nPrim, uint32_t prim,
                                             uint32_t entry)
{
	for (uint32_t j = 0; j < nPrim; ++j) {
		const size_t at = (size_t) slot * kClipFan + j;
		TriRaster R = P.clipR[at];
		TriAttr A = P.clipA[at];
		const uint32_t nt = A.pad;
		A.pad = 0;
		writeTri(P, R, A, nt, prim + j, entry);
		entry += nt;
	}
}

__device__ __forceinline__ void triStream(int prim, unsigned long long base, unsigned long long k, unsigned long long s[3])
{
	/* src/pipeline/topology.c:24-48 */
	if (prim == SRP_PRIM_TRIANGLES) { s[0] = base + 3 * k; s[1] = s[0] + 1; s[2] = s[0] + 2; }
	else if (prim == SRP_PRIM_TRIANGLE_STRIP) {
		const bool odd = (k & 1ull) != 0;
		s[0] = base + k + (odd ? 1 : 0);
		s[1] = base + k + (odd ? 0 : 1);
		s[2] = base + k + 2;
	} else { s[0] = base; s[1] = base + k + 1; s[2] = base + k + 2; }
}

__device__ __forceinline__ void lineStream(int prim, unsigned long long base, unsigned long long k,
                                           unsigned long long count, unsigned long long s[2])
{
	/* src/pipeline/topology.c:62-83 */
	if (prim == SRP_PRIM_LINES) { s[0] = base + 2 * k; s[1] = s[0] + 1; }
	else if (prim == SRP_PRIM_LINE_STRIP) { s[0] = base + k; s[1] = base + k + 1; }
	else { s[0] = base + k; s[1] = base + (k + 1) % count; }
}

__device__ __forceinline__ bool vertexIndex(const DrawParams& P, unsigned long long stream, uint32_t& vi)
{
	const unsigned long long v = P.indexSize ? fetchIndex(P, stream) : stream;
	if (v >= P.nVertices) { atomicOr(&P.ctr->errors, kErrBadIndex); return false; }
	vi = (uint32_t) v;
	return true;
}

__device__ __forceinline__ uint32_t vertexCode(const DrawParams& P, uint32_t vi)
{
	return P.codes[vi];
}

__device__ __forceinline__ SV loadSV(const DrawParams& P, uint32_t vi)
{
	const float4 a = P.vset0[vi], b = P.vset1[vi];
	SV v;
	v.s.nx = a.x; v.s.ny = a.y; v.s.sx = a.z; v.s.sy = a.w;
	v.s.c = b.x; v.s.iw = b.y; v.s.nz = b.z;
	v.ref = vi;
	return v;
}

__device__ __forceinline__ PV loadPV(const DrawParams& P, uint32_t vi)
{
	PV v;
	v.p = P.clip[vi];
	v.ref = vi;
	return v;
}

/* Status word of the decoupled look-back: flag (2 bits) | prims (30) | entries (32). */
__device__ __forceinline__ unsigned long long packStatus(unsigned long long flag, uint32_t prims, uint32_t entries)
{
	return (flag << 62) | ((unsigned long long) (prims & 0x3FFFFFFFu) << 32) | entries;
}

/* This thread's exclusive offset, (prims << 32) | entries, over the whole
 * launch in input order: a block scan, then a decoupled look-back over the
 * blocks in ticket order. The last block stores the totals in the counters.
 * Called by all threads of the block. */
__device__ __forceinline__ unsigned long long orderedOffset(const DrawParams& P, uint32_t bid, uint32_t nPrim,
                                                            uint32_t nEnt, unsigned long long* sWarp,
                                                            unsigned long long& sPrefix)
{
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	/* ---- block scan of (prims, entries) packed as one 64-bit sum */
	unsigned long long mine = ((unsigned long long) nPrim << 32) | nEnt;
	unsigned long long incl = mine;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
		if (lane >= o) incl += y;
	}
	if (lane == 31) sWarp[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		unsigned long long w = lane < kSetupThreads / 32 ? sWarp[lane] : 0ull;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, o);
			if (lane >= o) w += y;
		}
		if (lane < kSetupThreads / 32) sWarp[lane] = w;  /* inclusive over warps */
	}
	__syncthreads();
	const unsigned long long warpExcl = warp ? sWarp[warp - 1] : 0ull;
	const unsigned long long blockTotal = sWarp[kSetupThreads / 32 - 1];

	/* ---- decoupled look-back for the block's global offset */
	if (tid == 0) {
		const uint32_t aggP = (uint32_t) (blockTotal >> 32), aggE = (uint32_t) blockTotal;
		unsigned long long prefix = 0;
		if (bid == 0) {
			/* a failure-detection test withholds the first prefix: every
			 * later block's look-back then runs out (kErrSpin) */
			if (!(P.waitTest & kWaitTestSetup)) atomicExch(&P.lookback[0], packStatus(2, aggP, aggE));
		} else {
			atomicExch(&P.lookback[bid], packStatus(1, aggP, aggE));
			/* prims (bits 32..61) and entries (bits 0..31) summed as one word:
			 * the entry total stays below 2^32 (checked by the host) */
			const unsigned long long acc = lookBack<unsigned long long, 16>(
				P.lookback, (long long) bid - 1, 62, 0x3FFFFFFFFFFFFFFFull, &P.ctr->errors, spinBudget(P.spinLimit));
			const unsigned long long accP = acc >> 32, accE = acc & 0xFFFFFFFFull;
			if (accE + aggE > 0xFFFFFFFFull || accP + aggP > 0x3FFFFFFFull) atomicOr(&P.ctr->errors, kErrCapacity);
			atomicExch(&P.lookback[bid], packStatus(2, (uint32_t) (accP + aggP), (uint32_t) (accE + aggE)));
			prefix = (accP << 32) | (accE & 0xFFFFFFFFull);
		}
		sPrefix = prefix;
		if (bid == gridDim.x - 1) {
			P.ctr->prims = (prefix >> 32) + aggP;
			P.ctr->entries = (prefix & 0xFFFFFFFFull) + aggE;
		}
	}
	__syncthreads();
	return sPrefix + warpExcl + (incl - mine);
}

/* Filled triangles (millions per draw) run at kSetupBlocksPerSM; the other
 * modes, with their clip paths inline and far fewer primitives, at 6 blocks
 * per SM, whose registers hold them without spills. */
template <int MODE>
__global__ void __launch_bounds__(kSetupThreads, MODE == kTriFill ? kSetupBlocksPerSM : 6) k_setup(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	__shared__ uint32_t sBlock;
	__shared__ unsigned long long sWarp[kSetupThreads / 32];
	__shared__ unsigned long long sPrefix;
	/* an unclipped filled triangle's setup waits here across the scan, so
	 * that it holds no registers meanwhile */
	__shared__ TriRaster sR[MODE == kTriFill ? kSetupThreads : 1];
	__shared__ TriAttr sA[MODE == kTriFill ? kSetupThreads : 1];
	const int tid = threadIdx.x;
	if (tid == 0) sBlock = atomicAdd(&P.ctr->lookbackTicket, 1u);
	__syncthreads();
	const uint32_t bid = sBlock;
	const long long k = (long long) bid * kSetupThreads + tid;

	/* ---- phase A: assemble, clip, count */
	Assembly<MODE> as;
	as.nPoly = 0;
	as.clipped = false;
	bool live = k < P.nIn;
	if (live) {
		if (MODE == kPoints) {
			uint32_t vi;
			live = vertexIndex(P, P.start + (unsigned long long) k, vi);
			/* whole-point reject (src/pipeline/clipping.c:185-197): x < -w and
			 * x + w < 0 are the same test in fp32, so any outcode bit rejects */
			if (live) live = vertexCode(P, vi) == 0;
			if (live) as.sv[0] = loadSV(P, vi);
		} else if (MODE == kLines) {
			unsigned long long s[2];
			uint32_t vi[2];
			lineStream(P.prim, P.start, (unsigned long long) k, P.count, s);
			live = vertexIndex(P, s[0], vi[0]) && vertexIndex(P, s[1], vi[1]);
			if (live) {
				const uint32_t c0 = vertexCode(P, vi[0]), c1 = vertexCode(P, vi[1]);
				if ((c0 | c1) == 0) {
					as.sv[0] = loadSV(P, vi[0]);
					as.sv[1] = loadSV(P, vi[1]);
				} else if (c0 & c1) {
					live = false;
				} else {
					PV a = loadPV(P, vi[0]), b = loadPV(P, vi[1]);
					live = !clipLine(P, a, b);
					if (live) { as.sv[0] = fromClip(P.st, a); as.sv[1] = fromClip(P.st, b); }
				}
			}
		} else {
			unsigned long long s[3];
			uint32_t vi[3];
			triStream(P.prim, P.start, (unsigned long long) k, s);
			live = vertexIndex(P, s[0], vi[0]) && vertexIndex(P, s[1], vi[1]) && vertexIndex(P, s[2], vi[2]);
			if (live) {
				const uint32_t c0 = vertexCode(P, vi[0]), c1 = vertexCode(P, vi[1]), c2 = vertexCode(P, vi[2]);
				if (c0 & c1 & c2) live = false;
				else if ((c0 | c1 | c2) == 0) {
#pragma unroll
					for (int i = 0; i < 3; ++i) as.sv[i] = loadSV(P, vi[i]);
				} else {
					/* clipped by k_clip_prepass: read back its fan or its polygon */
					as.clipped = true;
					const uint32_t slot = P.clipSlot[k];
					if (slot >= P.clipPolyCap) { live = false; }
					else if constexpr (MODE == kTriFill) {
						as.slot = slot;
					} else {
						const uint32_t* poly = P.clipPolys + (size_t) slot * (1 + kMaxPoly);
						as.nPoly = (int) poly[0];
						for (int i = 0; i < as.nPoly && i < kMaxPoly; ++i) as.poly[i] = loadPV(P, poly[1 + i]);
						if (as.nPoly < 3) live = false;
					}
				}
			}
		}
	}
	uint32_t nPrim = 0, nEnt = 0;
	/* unclipped filled triangle: set up once, kept in shared memory across the scan */
	bool fOk = false;
	/* a line's run slots, kept across the scan */
	uint32_t lSlots = 0, lEnd = 0;
	if (live) {
		if (MODE == kPoints) {
			PointRec R;
			setupPoint(P.st, as.sv[0], R);
			nPrim = 1;
			nEnt = pointPairTiles(P.st, R);
		} else if (MODE == kLines) {
			LineRec L;
			setupLine(P.st, as.sv[0], as.sv[1], L);
			lineRunInfo(P.st, L);
			nPrim = 1;
			nEnt = lineSlots(L);
			lSlots = L.slots;
			lEnd = L.endPix;
		} else if (!as.clipped) {
			if (MODE == kTriFill) {
				TriRaster fR;
				TriAttr fA;
				fOk = setupTriangle(P.st, P.st.W, P.st.H, as.sv[0], as.sv[1], as.sv[2], fR, fA);
				if (fOk) {
					nPrim = 1;
					nEnt = triPairTiles(P.st, fR);
					sR[tid] = fR;
					sA[tid] = fA;
				}
			} else {
				handleTriangle<MODE>(P, as.sv[0], as.sv[1], as.sv[2], false, nPrim, nEnt);
			}
		} else if constexpr (MODE == kTriFill) {
			const uint2 fan = P.clipFan[as.slot];
			nPrim = fan.x;
			nEnt = fan.y;
		} else {
			const SV p0 = fromClip(P.st, as.poly[0]);
			for (int f = 1; f + 1 < as.nPoly; ++f)
				handleTriangle<MODE>(P, p0, fromClip(P.st, as.poly[f]), fromClip(P.st, as.poly[f + 1]), false, nPrim, nEnt);
		}
	}

	const unsigned long long base = orderedOffset(P, bid, nPrim, nEnt, sWarp, sPrefix);
	uint32_t primBase = (uint32_t) (base >> 32), entBase = (uint32_t) base;

	/* ---- phase C: write the survivors */
	if (!live) return;
	if (MODE == kPoints) {
		PointRec R;
		setupPoint(P.st, as.sv[0], R);
		if (primBase < P.primCap) {
			R.id = primBase;
			P.points[primBase] = R;
			int x0, y0, x1, y1;
			if (pointPairBox(P.st, R, x0, y0, x1, y1)) emitEntries(P, kKindPoint, primBase, entBase, x0, y0, x1, y1);
		} else atomicOr(&P.ctr->errors, kErrCapacity);
	} else if (MODE == kLines) {
		LineRec L;
		setupLine(P.st, as.sv[0], as.sv[1], L);
		L.slots = lSlots;
		L.endPix = lEnd;
		if (primBase < P.primCap) {
			L.id = primBase;
			L.fragBase = entBase;
			P.lines[primBase] = L;
		} else atomicOr(&P.ctr->errors, kErrCapacity);
	} else if (!as.clipped) {
		if (MODE == kTriFill) {
			if (fOk) {
				TriRaster fR = sR[tid];
				TriAttr fA = sA[tid];
				writeTri(P, fR, fA, nEnt, primBase, entBase);
			}
		} else {
			handleTriangle<MODE>(P, as.sv[0], as.sv[1], as.sv[2], true, primBase, entBase);
		}
	} else if constexpr (MODE == kTriFill) {
		writeClipFan(P, as.slot, nPrim, primBase, entBase);
	} else {
		const SV p0 = fromClip(P.st, as.poly[0]);
		for (int f = 1; f + 1 < as.nPoly; ++f)
			handleTriangle<MODE>(P, p0, fromClip(P.st, as.poly[f]), fromClip(P.st, as.poly[f + 1]), true, primBase, entBase);
	}
}

/* Clipping of the triangles that straddle a frustum plane, ahead of the
 * ordered setup: no ordering is needed to clip, so the long, divergent
 * Sutherland-Hodgman path runs here instead of inside the scan-coupled setup
 * blocks. The polygon (vertex count and vertex rows, new vertices included)
 * goes to a slot that k_setup reads back; for filled triangles the fan is
 * set up here as well, so that k_setup<kTriFill> only copies its records
 * (and carries no polygon, no stack frame and no spills). */
__global__ void __launch_bounds__(kSetupThreads, 16) k_clip_prepass(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	const long long k = (long long) blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= P.nIn) return;
	unsigned long long s[3];
	uint32_t vi[3];
	triStream(P.prim, P.start, (unsigned long long) k, s);
	if (!(vertexIndex(P, s[0], vi[0]) && vertexIndex(P, s[1], vi[1]) && vertexIndex(P, s[2], vi[2]))) return;
	const uint32_t c0 = vertexCode(P, vi[0]), c1 = vertexCode(P, vi[1]), c2 = vertexCode(P, vi[2]);
	if ((c0 & c1 & c2) || (c0 | c1 | c2) == 0) return;
	PV in[3] = { loadPV(P, vi[0]), loadPV(P, vi[1]), loadPV(P, vi[2]) };
	PV poly[kMaxPoly];
	const int n = clipPolygon(P, in, poly);
	const unsigned long long slot = atomicAdd(&P.ctr->clipTris, 1ull);
	if (slot >= P.clipPolyCap) { atomicOr(&P.ctr->errors, kErrCapacity); P.clipSlot[k] = 0xFFFFFFFFu; return; }
	uint32_t* out = P.clipPolys + (size_t) slot * (1 + kMaxPoly);
	out[0] = (uint32_t) n;
	for (int i = 0; i < n; ++i) out[1 + i] = poly[i].ref;
	if (P.st.polygonMode == SRP_POLYGON_MODE_FILL) setupClipFan<false>(P, (uint32_t) slot, poly, n, P.st.W, P.st.H);
	P.clipSlot[k] = (uint32_t) slot;
}

/* Lambda table of a big triangle: for every bbox row and every tile column,
 * the barycentrics the reference holds when its row walk reaches
 * max(minX, 8 * column) -- i.e. the exact serial chain. Each thread takes one
 * row and a run of up to 8 tile columns: it enters the run with the exact
 * jump-ahead (chain.h) and then adds dldx pixel by pixel, as the reference
 * does, storing the value at each column start. */
__device__ void fillLambdaTable(const DrawParams& P, const TriRaster& R, int first, int stride)
{
	if (R.table == kNoTable) return;
	const int rows = (int) R.maxY - (int) R.minY;
	const int c0 = (int) R.minX / kTile, c1 = ((int) R.maxX - 1) / kTile, ncols = c1 - c0 + 1;
	const int nseg = (ncols + 7) / 8;
	float* T = P.table + R.table;
	for (int idx = first; idx < rows * nseg; idx += stride) {
		const int r = idx / nseg, sg = idx % nseg;
		const int cs = c0 + sg * 8, ce = min(cs + 8, c1 + 1);
		int x = max((int) R.minX, cs * kTile);
		float l[3];
#pragma unroll
		for (int i = 0; i < 3; ++i)
			l[i] = srpChainAdd(srpChainAdd(R.l0[i], R.dy[i], (uint32_t) r), R.dx[i], (uint32_t) (x - R.minX));
		for (int c = cs; c < ce; ++c) {
			const int xt = max((int) R.minX, c * kTile);
			for (; x < xt; ++x)
#pragma unroll
				for (int i = 0; i < 3; ++i) l[i] = __fadd_rn(l[i], R.dx[i]);
			float* t = T + 3 * ((size_t) r * ncols + (c - c0));
			t[0] = l[0]; t[1] = l[1]; t[2] = l[2];
		}
	}
}

/* Entries of primitives covering more than kSmallEntries tiles: one block per
 * primitive writes its tiles row by row (and a triangle's lambda table). */
__global__ void k_big_entries(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (P.ctr->abort) return;
	const uint32_t nJobs = (uint32_t) min(P.ctr->bigJobs, (unsigned long long) P.bigCap);
	for (uint32_t j = blockIdx.x; j < nJobs; j += gridDim.x) {
		const uint4 job = P.bigJobs[j];
		/* the pixel box setup counted the job's pairs over */
		int x0, y0, x1, y1;
		if (job.z == kKindTri) triScissorBox(P.st, P.triR[job.x], x0, y0, x1, y1);
		else pointPairBox(P.st, P.points[job.x], x0, y0, x1, y1);
		const int tx0 = x0 / kTile, ty0 = y0 / kTile, ntx = x1 / kTile - tx0 + 1;
		for (uint32_t i = threadIdx.x; i < job.w; i += blockDim.x) {
			const uint32_t e = job.y + i;
			if (e >= P.entryCap) break;
			const int tx = tx0 + (int) (i % (uint32_t) ntx), ty = ty0 + (int) (i / (uint32_t) ntx);
			P.keys[e] = (uint32_t) (ty * P.st.tilesX + tx);
			P.vals[e] = job.x;
		}
	}
}

/* Lambda tables of all big triangles: blockIdx.y walks the jobs, the
 * blockIdx.x blocks of a job share its (row, column-run) work items. */
__global__ void k_lambda_tables(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (P.ctr->abort) return;
	const uint32_t nJobs = (uint32_t) min(P.ctr->bigJobs, (unsigned long long) P.bigCap);
	for (uint32_t j = blockIdx.y; j < nJobs; j += gridDim.y) {
		const uint4 job = P.bigJobs[j];
		if (job.z != kKindTri) continue;
		fillLambdaTable(P, P.triR[job.x], blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
	}
}

/* Steps [s0, s1) of line i's DDA, exactly as the reference walks them
 * (fp32 accumulators, round half away from zero; src/raster/line.c:34-77),
 * from the accumulators (x, y, t) at step s0. Steps whose pixel fails the
 * scissor test or falls outside the framebuffer are dropped
 * (src/raster/fragment.c:63-75); the others form runs (see lineRunInfo),
 * written to slots slot0.. of the pair arrays, at most nSlots of them; the
 * slots left over get the key one past the last tile, which sorts them out.
 * Returns the steps that passed the scissor test. */
__device__ unsigned long long walkLineRuns(const DrawParams& P, const LineRec& L, uint32_t i, uint32_t s0, uint32_t s1,
                                           float x, float y, float t, uint32_t slot0, uint32_t nSlots)
{
	unsigned long long passed = 0;
	const uint32_t invalid = (uint32_t) (P.st.tilesX * P.st.tilesY);
	const unsigned long long size = (unsigned long long) P.st.W * (unsigned long long) P.st.H;
	const bool inside = (L.slots & kLineInside) != 0;
	uint32_t used = 0, runKey = invalid, runN = 0;
	auto flush = [&]() {
		if (runN) {
			const uint32_t k = slot0 + used;
			if (used < nSlots && k < P.entryCap) {
				P.keys[k] = runKey;
				P.vals[k] = k | (runN << kRunCountShift);
			}
			++used;
		}
		runN = 0;
	};
	for (uint32_t s = s0; s < s1; ++s) {
		const int px = (int) roundf(x), py = (int) roundf(y);
		uint32_t key = invalid;
		if (scissorPass(P.st, px, py)) {
			++passed;  /* counted as the reference's fragments are, before the framebuffer bound */
			if (inside) {
				/* every step of the line lands in the framebuffer (lineRunInfo):
				 * the pixel is (px, py) itself, no row wraps */
				key = ((uint32_t) py / kTile) * (uint32_t) P.st.tilesX + (uint32_t) px / kTile;
			} else {
				const unsigned long long idx = (unsigned long long) (long long) py * (unsigned long long) P.st.W
				                             + (unsigned long long) (long long) px;
				if (idx < size) {
					const uint32_t gx = (uint32_t) (idx % (unsigned long long) P.st.W);
					const uint32_t gy = (uint32_t) (idx / (unsigned long long) P.st.W);
					key = (gy / kTile) * (uint32_t) P.st.tilesX + gx / kTile;
				}
			}
		}
		if (key != runKey || runN == kRunMaxCount) {
			flush();
			runKey = key;
		}
		if (key != invalid) {
			const uint32_t k = slot0 + used;
			if (used < nSlots && k < P.entryCap) {
				const unsigned long long rec = (unsigned long long) k * kRunFrags + runN;
				if (rec < P.fragCap) {
					LineFrag F;
					F.depth = __fadd_rn(__fmul_rn(L.c[0], __fsub_rn(1.0f, t)), __fmul_rn(L.c[1], t));
					F.t = t; F.line = i; F.px = (int16_t) px; F.py = (int16_t) py;
					P.frags[rec] = F;
				}
			}
			++runN;
		}
		x = __fadd_rn(x, L.xInc);
		y = __fadd_rn(y, L.yInc);
		t = __fadd_rn(t, L.tInc);
	}
	flush();
	for (uint32_t u = used; u < nSlots; ++u) {
		const uint32_t k = slot0 + u;
		if (k < P.entryCap) { P.keys[k] = invalid; P.vals[k] = 0; }
	}
	return passed;
}

/* One thread per line; lines longer than kShortLine steps are queued for
 * k_line_frags_long. */
__global__ void k_line_frags(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (P.ctr->abort) return;
	const uint32_t nLines = (uint32_t) min(P.ctr->prims, (unsigned long long) P.primCap);
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	unsigned long long passed = 0;
	if (i < nLines) {
		const LineRec L = P.lines[i];
		const uint32_t total = (uint32_t) L.steps + 1u;
		if (total > kShortLine) {
			const unsigned long long j = atomicAdd(&P.ctr->lineFrags, 1ull);
			if (j < P.bigCap) P.bigJobs[j].x = i;
		} else {
			passed = walkLineRuns(P, L, i, 0, total, L.x0, L.y0, 0.0f, L.fragBase, lineSlots(L));
		}
	}
	for (int o = 16; o; o >>= 1) passed += __shfl_xor_sync(0xFFFFFFFFu, passed, o);
	if ((threadIdx.x & 31) == 0 && passed) atomicAdd(&P.ctr->fragments, passed);
}

/* Long lines: one warp per line, lane l walks a contiguous segment of steps
 * into its share of the line's slots. A lane's share is bounded by the tile
 * distance from its first pixel to the next lane's first pixel (the far
 * pixel E of lineRunInfo for the last lane), + 1, or by its step count
 * when not every step of the line lands in the framebuffer (lineRunInfo);
 * an exclusive scan of the shares places them, and the last lane clears
 * the slots beyond them. */
__global__ void k_line_frags_long(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (P.ctr->abort) return;
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t nLong = (uint32_t) min(P.ctr->lineFrags, (unsigned long long) P.bigCap);
	const uint32_t warps = gridDim.x * (blockDim.x / 32);
	for (uint32_t q = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); q < nLong; q += warps) {
		const uint32_t i = P.bigJobs[q].x;
		const LineRec L = P.lines[i];
		const uint32_t total = (uint32_t) L.steps + 1u;
		const uint32_t seg = (total + 31u) / 32u;
		const uint32_t s0 = min(lane * seg, total), s1 = min(s0 + seg, total);
		const float x = srpChainAdd(L.x0, L.xInc, s0), y = srpChainAdd(L.y0, L.yInc, s0);
		const float t = srpChainAdd(0.0f, L.tInc, s0);
		const int px = (int) roundf(x), py = (int) roundf(y);
		int nx = __shfl_down_sync(0xFFFFFFFFu, px, 1), ny = __shfl_down_sync(0xFFFFFFFFu, py, 1);
		if (lane == 31) { nx = (int) (int16_t) (L.endPix & 0xFFFFu); ny = (int) (int16_t) (L.endPix >> 16); }
		uint32_t mine = s1 - s0;
		if ((L.slots & kLineInside) && mine) {
			const uint32_t d = tileDistance(px, py, nx, ny) + 1u;
			if (d < mine) mine = d;
		}
		uint32_t incl = mine;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
			if (lane >= (uint32_t) o) incl += v;
		}
		unsigned long long passed = walkLineRuns(P, L, i, s0, s1, x, y, t, L.fragBase + incl - mine, mine);
		if (lane == 31) {
			const uint32_t invalid = (uint32_t) (P.st.tilesX * P.st.tilesY);
			for (uint32_t u = incl; u < lineSlots(L); ++u) {
				const uint32_t k = L.fragBase + u;
				if (k < P.entryCap) { P.keys[k] = invalid; P.vals[k] = 0; }
			}
		}
		for (int o = 16; o; o >>= 1) passed += __shfl_xor_sync(0xFFFFFFFFu, passed, o);
		if (lane == 0 && passed) atomicAdd(&P.ctr->fragments, passed);
	}
}

/* Runs back to fragments, after the sort: the fragment counts of the sorted
 * runs are scanned (per block of kRunBlock, then over the blocks), and every
 * run writes its fragments' record numbers to fragVals in sorted order and,
 * if it is the first or last run of its tile, the tile's fragment range, so
 * that the resolve and shading kernels see one item per fragment in (tile,
 * line, step) order. */
constexpr int kRunBlock = 1024;

__device__ __forceinline__ uint32_t runCount(uint32_t v) { return v >> kRunCountShift; }

__global__ void __launch_bounds__(kRunBlock) k_run_sums(const __grid_constant__ DrawParams P, const uint32_t* vals)
{
	gridDepSync();
	__shared__ uint32_t sw[kRunBlock / 32];
	const uint32_t n = (uint32_t) min(P.ctr->entries, (unsigned long long) P.entryCap);
	const uint32_t i = blockIdx.x * kRunBlock + threadIdx.x;
	uint32_t c = (i < n && !P.ctr->abort) ? runCount(vals[i]) : 0u;
	for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
	if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x < 32) {
		uint32_t v = sw[threadIdx.x];
		for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
		if (threadIdx.x == 0) P.runSums[blockIdx.x] = v;
	}
}

/* Exclusive scan of the nb block sums in place; runSums[nb] = the total. */
__global__ void __launch_bounds__(kRunBlock) k_run_scan(const __grid_constant__ DrawParams P, uint32_t nb)
{
	gridDepSync();
	__shared__ uint32_t sw[kRunBlock / 32];
	__shared__ uint32_t carry;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (threadIdx.x == 0) carry = 0;
	__syncthreads();
	for (uint32_t b0 = 0; b0 < nb; b0 += kRunBlock) {
		const uint32_t b = b0 + threadIdx.x;
		const uint32_t v = b < nb ? P.runSums[b] : 0u;
		uint32_t incl = v;
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
			if (lane >= o) incl += y;
		}
		if (lane == 31) sw[warp] = incl;
		__syncthreads();
		if (warp == 0) {
			uint32_t w = sw[lane];
			for (int o = 1; o < 32; o <<= 1) {
				const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
				if (lane >= o) w += y;
			}
			sw[lane] = w;
		}
		__syncthreads();
		const uint32_t excl = carry + (warp ? sw[warp - 1] : 0u) + incl - v;
		if (b < nb) P.runSums[b] = excl;
		__syncthreads();
		if (threadIdx.x == kRunBlock - 1) carry = excl + v;
		__syncthreads();
	}
	if (threadIdx.x == 0) P.runSums[nb] = carry;
}

__global__ void __launch_bounds__(kRunBlock) k_run_expand(const __grid_constant__ DrawParams P, const uint32_t* keys,
                                                          const uint32_t* vals, uint32_t numTiles)
{
	gridDepSync();
	__shared__ uint32_t sw[kRunBlock / 32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t n = (uint32_t) min(P.ctr->entries, (unsigned long long) P.entryCap);
	const uint32_t i = blockIdx.x * kRunBlock + threadIdx.x;
	const uint32_t v = (i < n && !P.ctr->abort) ? vals[i] : 0u;
	const uint32_t c = runCount(v);
	uint32_t incl = c;
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
		if (lane >= o) incl += y;
	}
	if (lane == 31) sw[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		uint32_t w = sw[lane];
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
			if (lane >= o) w += y;
		}
		sw[lane] = w;
	}
	__syncthreads();
	const uint32_t off = P.runSums[blockIdx.x] + (warp ? sw[warp - 1] : 0u) + incl - c;
	if (c == 0) return;
	const uint32_t k = v & ((1u << kRunCountShift) - 1u);
	for (uint32_t j = 0; j < c; ++j)
		if (off + j < P.fragCap) P.fragVals[off + j] = k * kRunFrags + j;
	const uint32_t key = keys[i];
	if (key >= numTiles) return;
	if (i == 0 || keys[i - 1] != key) P.tileStart[key] = off;
	if (i + 1 == n || keys[i + 1] != key) P.tileEnd[key] = off + c;
}

/* ============================================================ multi-draw */

/* A multi-draw pass (srpGpuDrawBatch) runs many independent triangle draws,
 * each into its own framebuffer, through one set of launches. Input
 * primitives, vertex rows, tiles and (tile, item) pairs are numbered
 * globally over the pass; each work item finds its draw by a binary search
 * over the pass's prefix arrays. Within a draw the order is the draw's own
 * submission order, exactly as for a single draw, so every draw renders as
 * if it had been issued alone. */

/* The draw d holding position x: prefix[d] <= x < prefix[d + 1]. Empty
 * draws share their successor's start and are never returned. */
__device__ __forceinline__ uint32_t drawOf(const uint32_t* prefix, uint32_t n, uint32_t x)
{
	uint32_t lo = 0, hi = n;
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (__ldg(prefix + mid) <= x) lo = mid; else hi = mid;
	}
	return lo;
}

/* Vertex shading of every vertex of every draw of the pass. Blocks are
 * handed out per draw (blkPrefix), so a block stages one contiguous run of
 * one vertex buffer exactly as k_vertex does. */
template <int VS>
__global__ void __launch_bounds__(kVertexThreads) k_vertex_multi(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	extern __shared__ uint32_t stage[];
	const uint32_t d = drawOf(P.blkPrefix, P.nDraws, blockIdx.x);
	const DrawDesc& D = P.draws[d];
	const unsigned long long vb = (unsigned long long) (blockIdx.x - P.blkPrefix[d]) * kVertexThreads;
	const unsigned long long nV = D.nVertices;
	if (vb >= nV) return;
	const unsigned long long vend = vb + kVertexThreads < nV ? vb + kVertexThreads : nV;
	const int stride = D.stride;
	const unsigned long long bytes = (vend - vb) * (unsigned long long) stride;
	const unsigned char* src = D.vertices + vb * (unsigned long long) stride;
	if ((stride & 3) == 0) {
		const uint32_t* w = (const uint32_t*) src;
		for (unsigned long long i = threadIdx.x; i < bytes / 4; i += kVertexThreads) stage[i] = __ldg(w + i);
	} else {
		unsigned char* sb = (unsigned char*) stage;
		for (unsigned long long i = threadIdx.x; i < bytes; i += kVertexThreads) sb[i] = __ldg(src + i);
	}
	__syncthreads();
	const unsigned long long v = vb + threadIdx.x;
	if (v >= vend) return;
	uint32_t vtx[kMaxVertexWords];
	const unsigned char* rec = (const unsigned char*) stage + (unsigned long long) threadIdx.x * stride;
	const int words = (stride + 3) / 4 < kMaxVertexWords ? (stride + 3) / 4 : kMaxVertexWords;
#pragma unroll
	for (int k = 0; k < kMaxVertexWords; ++k) vtx[k] = 0;
	if ((stride & 3) == 0) {
#pragma unroll
		for (int k = 0; k < kMaxVertexWords; ++k)
			if (k < words) vtx[k] = ((const uint32_t*) rec)[k];
	} else {
		memcpy(vtx, rec, stride < 4 * kMaxVertexWords ? stride : 4 * kMaxVertexWords);
	}
	uint32_t out[kMaxVaryingWords];
#pragma unroll
	for (int k = 0; k < kMaxVaryingWords; ++k) out[k] = 0;
	SRPVertexShaderIn in;
	in.uniform = (SRPUniform*) D.uniform;
	in.vertex = (SRPVertex*) vtx;
	in.vertexID = (size_t) v;
	SRPVertexShaderOut o;
	o.clipPosition[0] = o.clipPosition[1] = o.clipPosition[2] = o.clipPosition[3] = 0.0f;
	o.varyings = (SRPVarying*) out;
	runVS<VS>(&in, &o);
	const float4 clip = make_float4(o.clipPosition[0], o.clipPosition[1], o.clipPosition[2], o.clipPosition[3]);
	const unsigned long long row = P.vPrefix[d] + v;
	P.clip[row] = clip;
	const uint32_t code = outcode(clip);
	P.codes[row] = (uint8_t) code;
	if (code == 0) {
		const VSet vs = vertexSetup(D.W, D.H, clip);
		P.vset0[row] = make_float4(vs.nx, vs.ny, vs.sx, vs.sy);
		P.vset1[row] = make_float4(vs.c, vs.iw, vs.nz, __uint_as_float(0u));
	}
	const int nw = P.L.nWords;
	uint32_t* dst = P.vary + row * (unsigned long long) nw;
#pragma unroll
	for (int k = 0; k < kMaxVaryingWords; ++k)
		if (k < nw) dst[k] = out[k];
}

/* Vertex row of stream position `stream` of draw D (rows of the pass start
 * at rowBase for this draw). */
__device__ __forceinline__ bool vertexIndexD(const DrawParams& P, const DrawDesc& D, uint32_t rowBase,
                                             unsigned long long stream, uint32_t& vi)
{
	const unsigned long long v = D.indexSize ? fetchIndexRaw(D.indices, D.indexSize, stream) : stream;
	if (v >= D.nVertices) { atomicOr(&P.ctr->errors, kErrBadIndex); return false; }
	vi = rowBase + (uint32_t) v;
	return true;
}

/* Input triangle k of the pass: its draw and its three vertex rows. */
__device__ __forceinline__ bool triangleOfPass(const DrawParams& P, uint32_t k, uint32_t& d, uint32_t vi[3],
                                               unsigned long long& local)
{
	d = drawOf(P.inPrefix, P.nDraws, k);
	const DrawDesc& D = P.draws[d];
	local = (unsigned long long) (k - P.inPrefix[d]);
	unsigned long long s[3];
	triStream(D.prim, D.start, local, s);
	const uint32_t rb = P.vPrefix[d];
	return vertexIndexD(P, D, rb, s[0], vi[0]) && vertexIndexD(P, D, rb, s[1], vi[1]) &&
	       vertexIndexD(P, D, rb, s[2], vi[2]);
}

/* Clip pre-pass of a pass (see k_clip_prepass). */
__global__ void __launch_bounds__(kSetupThreads, 16) k_clip_prepass_multi(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	const long long k = (long long) blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= P.nIn) return;
	uint32_t d, vi[3];
	unsigned long long local;
	if (!triangleOfPass(P, (uint32_t) k, d, vi, local)) return;
	const uint32_t c0 = vertexCode(P, vi[0]), c1 = vertexCode(P, vi[1]), c2 = vertexCode(P, vi[2]);
	if ((c0 & c1 & c2) || (c0 | c1 | c2) == 0) return;
	PV in[3] = { loadPV(P, vi[0]), loadPV(P, vi[1]), loadPV(P, vi[2]) };
	PV poly[kMaxPoly];
	const int n = clipPolygon(P, in, poly);
	const unsigned long long slot = atomicAdd(&P.ctr->clipTris, 1ull);
	if (slot >= P.clipPolyCap) { atomicOr(&P.ctr->errors, kErrCapacity); P.clipSlot[k] = 0xFFFFFFFFu; return; }
	uint32_t* out = P.clipPolys + (size_t) slot * (1 + kMaxPoly);
	out[0] = (uint32_t) n;
	for (int i = 0; i < n; ++i) out[1 + i] = poly[i].ref;
	const DrawDesc& D = P.draws[d];
	setupClipFan<true>(P, (uint32_t) slot, poly, n, D.W, D.H);
	P.clipSlot[k] = (uint32_t) slot;
}

/* Pairs of a triangle of draw d: keys are global tile numbers of the pass;
 * big triangles are queued with the draw in place of the kind. */
__device__ void emitEntriesMulti(const DrawParams& P, uint32_t d, int tilesX, uint32_t tileBase, uint32_t item,
                                 uint32_t base, int x0, int y0, int x1, int y1)
{
	const uint32_t n = tileCount(x0, y0, x1 + 1, y1 + 1);
	if (n == 0) return;
	if (n <= (uint32_t) kSmallEntries) {
		uint32_t e = base;
		for (int ty = y0 / kTile; ty <= y1 / kTile; ++ty)
			for (int tx = x0 / kTile; tx <= x1 / kTile; ++tx, ++e)
				if (e < P.entryCap) { P.keys[e] = tileBase + (uint32_t) (ty * tilesX + tx); P.vals[e] = item; }
		if (base + n > P.entryCap) atomicOr(&P.ctr->errors, kErrCapacity);
	} else {
		const unsigned long long j = atomicAdd(&P.ctr->bigJobs, 1ull);
		if (j < P.bigCap) P.bigJobs[j] = make_uint4(item, base, d, n);
		else atomicOr(&P.ctr->errors, kErrCapacity);
	}
}

__device__ __forceinline__ void writeTriMulti(const DrawParams& P, uint32_t d, int tilesX, uint32_t tileBase,
                                              TriRaster& R, TriAttr& A, uint32_t nt, uint32_t prim, uint32_t entry)
{
	if (nt > (uint32_t) kSmallEntries) {
		const int cols = ((int) R.maxX - 1) / kTile - (int) R.minX / kTile + 1;
		const unsigned long long words = 3ull * (unsigned long long) (R.maxY - R.minY) * (unsigned long long) cols;
		const unsigned long long off = atomicAdd(&P.ctr->tableWords, words);
		if (off + words <= P.tableCap && off < 0xFFFFFFFFull) R.table = (uint32_t) off;
	}
	if (prim < P.primCap) {
		A.id = prim;
		P.triR[prim] = R;
		P.triA[prim] = A;
		emitEntriesMulti(P, d, tilesX, tileBase, prim, entry, R.minX, R.minY, (int) R.maxX - 1, (int) R.maxY - 1);
	} else atomicOr(&P.ctr->errors, kErrCapacity);
}

/* Ordered setup of a pass (filled triangles): as k_setup<kTriFill>, with the
 * draw's framebuffer size and tile grid. The first input triangle of every
 * draw records the number of surviving primitives before the draw, from
 * which primitive ids local to the draw are recovered. */
/* 8 blocks per SM: 62 registers without spills (at 10 per SM the kernel
 * spilled 100 bytes; the batch's setup stage measured 9.45 -> 9.22 ms) */
__global__ void __launch_bounds__(kSetupThreads, 8) k_setup_multi(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	__shared__ uint32_t sBlock;
	__shared__ unsigned long long sWarp[kSetupThreads / 32];
	__shared__ unsigned long long sPrefix;
	__shared__ TriRaster sR[kSetupThreads];
	__shared__ TriAttr sA[kSetupThreads];
	const int tid = threadIdx.x;
	if (tid == 0) sBlock = atomicAdd(&P.ctr->lookbackTicket, 1u);
	__syncthreads();
	const uint32_t bid = sBlock;
	const long long k = (long long) bid * kSetupThreads + tid;

	bool live = k < P.nIn, clipped = false, first = false;
	uint32_t d = 0;
	int W = 0, H = 0, tilesX = 0;
	uint32_t tileBase = 0;
	SV sv[3];
	uint32_t slot = 0;
	if (live) {
		uint32_t vi[3];
		unsigned long long local;
		live = triangleOfPass(P, (uint32_t) k, d, vi, local);
		first = local == 0;
		const DrawDesc& D = P.draws[d];
		W = D.W; H = D.H; tilesX = D.tilesX;
		tileBase = P.tPrefix[d];
		if (live) {
			const uint32_t c0 = vertexCode(P, vi[0]), c1 = vertexCode(P, vi[1]), c2 = vertexCode(P, vi[2]);
			if (c0 & c1 & c2) live = false;
			else if ((c0 | c1 | c2) == 0) {
#pragma unroll
				for (int i = 0; i < 3; ++i) sv[i] = loadSV(P, vi[i]);
			} else {
				/* clipped: its fan was set up by k_clip_prepass_multi */
				clipped = true;
				slot = P.clipSlot[k];
				if (slot >= P.clipPolyCap) live = false;
			}
		}
	}
	uint32_t nPrim = 0, nEnt = 0;
	bool fOk = false;
	if (live) {
		if (!clipped) {
			TriRaster fR;
			TriAttr fA;
			fOk = setupTriangle(P.st, W, H, sv[0], sv[1], sv[2], fR, fA);
			if (fOk) {
				nPrim = 1;
				nEnt = tileCount(fR.minX, fR.minY, fR.maxX, fR.maxY);
				sR[tid] = fR;
				sA[tid] = fA;
			}
		} else {
			const uint2 fan = P.clipFan[slot];
			nPrim = fan.x;
			nEnt = fan.y;
		}
	}
	const unsigned long long base = orderedOffset(P, bid, nPrim, nEnt, sWarp, sPrefix);
	uint32_t primBase = (uint32_t) (base >> 32), entBase = (uint32_t) base;
	if (first) P.primPrefix[d] = primBase;
	if (!live) return;
	if (!clipped) {
		if (fOk) {
			TriRaster fR = sR[tid];
			TriAttr fA = sA[tid];
			writeTriMulti(P, d, tilesX, tileBase, fR, fA, nEnt, primBase, entBase);
		}
	} else {
		for (uint32_t j = 0; j < nPrim; ++j) {
			const size_t at = (size_t) slot * kClipFan + j;
			TriRaster R = P.clipR[at];
			TriAttr A = P.clipA[at];
			const uint32_t nt = A.pad;
			A.pad = 0;
			writeTriMulti(P, d, tilesX, tileBase, R, A, nt, primBase + j, entBase);
			entBase += nt;
		}
	}
}

/* k_big_entries for a pass: the job's third word is its draw. */
__global__ void k_big_entries_multi(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (P.ctr->abort) return;
	const uint32_t nJobs = (uint32_t) min(P.ctr->bigJobs, (unsigned long long) P.bigCap);
	for (uint32_t j = blockIdx.x; j < nJobs; j += gridDim.x) {
		const uint4 job = P.bigJobs[j];
		const TriRaster& R = P.triR[job.x];
		const int x0 = R.minX, y0 = R.minY, x1 = (int) R.maxX - 1;
		const int tilesX = P.draws[job.z].tilesX;
		const uint32_t tileBase = P.tPrefix[job.z];
		const int tx0 = x0 / kTile, ty0 = y0 / kTile, ntx = x1 / kTile - tx0 + 1;
		for (uint32_t i = threadIdx.x; i < job.w; i += blockDim.x) {
			const uint32_t e = job.y + i;
			if (e >= P.entryCap) break;
			const int tx = tx0 + (int) (i % (uint32_t) ntx), ty = ty0 + (int) (i / (uint32_t) ntx);
			P.keys[e] = tileBase + (uint32_t) (ty * tilesX + tx);
			P.vals[e] = job.x;
		}
	}
}

/* Lambda tables of a pass's big triangles (every job is a triangle). */
__global__ void k_lambda_tables_multi(const __grid_constant__ DrawParams P)
{
	gridDepSync();
	if (P.ctr->abort) return;
	const uint32_t nJobs = (uint32_t) min(P.ctr->bigJobs, (unsigned long long) P.bigCap);
	for (uint32_t j = blockIdx.y; j < nJobs; j += gridDim.y) {
		const uint4 job = P.bigJobs[j];
		fillLambdaTable(P, P.triR[job.x], blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
	}
}

/* ------------------------------------------------------------ launchers */

void launchReset(const DrawParams& P, cudaStream_t s) { pdlLaunch(k_reset, 1, 32, 0, s, P); }

void launchIndexRange(const DrawParams& P, cudaStream_t s)
{
	/* 16-byte words of the range, two per thread */
	const unsigned long long words = (P.count * (unsigned long long) P.indexSize + 31) / 16;
	unsigned long long blocks = (words + 511) / 512;
	if (blocks > 152 * 8) blocks = 152 * 8;
	if (blocks < 1) blocks = 1;
	pdlLaunch(k_index_range, (unsigned) blocks, 256, 0, s, P);
}

void launchVertex(const DrawParams& P, unsigned long long first, unsigned long long n, cudaStream_t s)
{
	const unsigned blocks = (unsigned) ((n + kVertexThreads - 1) / kVertexThreads);
	if (!blocks) return;
	const size_t smem = (size_t) kVertexThreads * P.stride + 16;
	switch (P.vsId) {
	case SRP_GPU_VS_WORLD:
		cudaFuncSetAttribute(k_vertex<SRP_GPU_VS_WORLD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
		pdlLaunch(k_vertex<SRP_GPU_VS_WORLD>, blocks, kVertexThreads, smem, s, P, first, n);
		break;
	case SRP_GPU_VS_BYTES:
		cudaFuncSetAttribute(k_vertex<SRP_GPU_VS_BYTES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
		pdlLaunch(k_vertex<SRP_GPU_VS_BYTES>, blocks, kVertexThreads, smem, s, P, first, n);
		break;
	default:
		cudaFuncSetAttribute(k_vertex<SRP_GPU_VS_TRANSFORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
		pdlLaunch(k_vertex<SRP_GPU_VS_TRANSFORM>, blocks, kVertexThreads, smem, s, P, first, n);
		break;
	}
}

void launchSetup(const DrawParams& P, cudaStream_t s)
{
	const unsigned blocks = (unsigned) ((P.nIn + kSetupThreads - 1) / kSetupThreads);
	if (!blocks) return;
	const bool tri = P.prim == SRP_PRIM_TRIANGLES || P.prim == SRP_PRIM_TRIANGLE_STRIP || P.prim == SRP_PRIM_TRIANGLE_FAN;
	if (tri && P.st.polygonMode == SRP_POLYGON_MODE_LINE) pdlLaunch(k_setup<kTriLine>, blocks, kSetupThreads, 0, s, P);
	else if (tri && P.st.polygonMode == SRP_POLYGON_MODE_POINT) pdlLaunch(k_setup<kTriPoint>, blocks, kSetupThreads, 0, s, P);
	else if (tri) pdlLaunch(k_setup<kTriFill>, blocks, kSetupThreads, 0, s, P);
	else if (P.prim == SRP_PRIM_POINTS) pdlLaunch(k_setup<kPoints>, blocks, kSetupThreads, 0, s, P);
	else pdlLaunch(k_setup<kLines>, blocks, kSetupThreads, 0, s, P);
}

void launchClipPrepass(const DrawParams& P, cudaStream_t s)
{
	const unsigned blocks = (unsigned) ((P.nIn + kSetupThreads - 1) / kSetupThreads);
	if (blocks) pdlLaunch(k_clip_prepass, blocks, kSetupThreads, 0, s, P);
}

/* Grids for a job count the device holds: sized from the hint, any size is
 * correct since the kernels stride over the jobs. */
static unsigned bigBlocks(uint32_t hint) { return hint < 64u ? 64u : (hint < 152u * 16u ? hint : 152u * 16u); }
static unsigned tableRows(uint32_t hint) { return hint < 64u ? 64u : (hint < 65535u ? hint : 65535u); }

void launchCheck(const DrawParams& P, cudaStream_t s) { pdlLaunch(k_check, 1, 32, 0, s, P); }

void launchBigEntries(const DrawParams& P, uint32_t jobsHint, cudaStream_t s)
{
	pdlLaunch(k_big_entries, bigBlocks(jobsHint), 256, 0, s, P);
}

void launchLambdaTables(const DrawParams& P, uint32_t jobsHint, cudaStream_t s)
{
	pdlLaunch(k_lambda_tables, dim3(8, tableRows(jobsHint)), 256, 0, s, P);
}

void launchLineFrags(const DrawParams& P, cudaStream_t s)
{
	if (!P.primCap) return;
	pdlLaunch(k_line_frags, (P.primCap + 127) / 128, 128, 0, s, P);
	pdlLaunch(k_line_frags_long, 152 * 8, 128, 0, s, P);
}

uint32_t runSumWords(uint32_t entryCap) { return (entryCap + kRunBlock - 1) / kRunBlock + 2; }

void launchRunExpand(const DrawParams& P, const uint32_t* keys, const uint32_t* vals, uint32_t numTiles, cudaStream_t s)
{
	if (!P.entryCap) return;
	const uint32_t nb = (P.entryCap + kRunBlock - 1) / kRunBlock;
	pdlLaunch(k_run_sums, nb, kRunBlock, 0, s, P, vals);
	pdlLaunch(k_run_scan, 1, kRunBlock, 0, s, P, nb);
	pdlLaunch(k_run_expand, nb, kRunBlock, 0, s, P, keys, vals, numTiles);
}

void launchVertexMulti(const DrawParams& P, uint32_t blocks, int maxStride, cudaStream_t s)
{
	if (!blocks) return;
	const size_t smem = (size_t) kVertexThreads * maxStride + 16;
	switch (P.vsId) {
	case SRP_GPU_VS_WORLD:
		cudaFuncSetAttribute(k_vertex_multi<SRP_GPU_VS_WORLD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
		pdlLaunch(k_vertex_multi<SRP_GPU_VS_WORLD>, blocks, kVertexThreads, smem, s, P);
		break;
	case SRP_GPU_VS_BYTES:
		cudaFuncSetAttribute(k_vertex_multi<SRP_GPU_VS_BYTES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
		pdlLaunch(k_vertex_multi<SRP_GPU_VS_BYTES>, blocks, kVertexThreads, smem, s, P);
		break;
	default:
		cudaFuncSetAttribute(k_vertex_multi<SRP_GPU_VS_TRANSFORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
		pdlLaunch(k_vertex_multi<SRP_GPU_VS_TRANSFORM>, blocks, kVertexThreads, smem, s, P);
		break;
	}
}

void launchClipPrepassMulti(const DrawParams& P, cudaStream_t s)
{
	const unsigned blocks = (unsigned) ((P.nIn + kSetupThreads - 1) / kSetupThreads);
	if (blocks) pdlLaunch(k_clip_prepass_multi, blocks, kSetupThreads, 0, s, P);
}

void launchSetupMulti(const DrawParams& P, cudaStream_t s)
{
	const unsigned blocks = (unsigned) ((P.nIn + kSetupThreads - 1) / kSetupThreads);
	if (blocks) pdlLaunch(k_setup_multi, blocks, kSetupThreads, 0, s, P);
}

void launchBigEntriesMulti(const DrawParams& P, uint32_t jobsHint, cudaStream_t s)
{
	pdlLaunch(k_big_entries_multi, bigBlocks(jobsHint), 256, 0, s, P);
}

void launchLambdaTablesMulti(const DrawParams& P, uint32_t jobsHint, cudaStream_t s)
{
	pdlLaunch(k_lambda_tables_multi, dim3(8, tableRows(jobsHint)), 256, 0, s, P);
}

}  // namespace srpg
