/* CPU oracle: a restatement of kitrofimov/srp's draw path in plain C.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker the GPU path is compared
 * against (tests, the smoke check and the CPU-baseline leg of bench.py); it is
 * never linked into, loaded by or called from the product library.
 *
 * It implements the same public API (include/srp/*.h) single-threaded on the
 * host and follows the reference's arithmetic operation by operation, because
 * coverage, depth and stencil must agree bit for bit: fp32 without
 * contraction (build with -ffp-contract=off), the reference's double-precision
 * spots kept in double, the serial barycentric add chain, the top-left-rule
 * pairing quirk, post-clip/post-cull primitive numbering. Each function names
 * the reference file:line range it restates. Memory is plain malloc instead of
 * the reference's arena (src/memory/arena.c); that changes no result.
 *
 * The restatement is pinned against the reference's own golden images and
 * against the reference library built from source (see oracle/Makefile). */
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "srp/srp.h"
#include "srp/mat.h"
#include "../srp_gb300/csrc/imageio.h"

/* ------------------------------------------------------------------ utils */

#define EPS_DOUBLE 1e-9
/* ROUGHLY_ZERO(x) is fabs((double) x) <= 1e-9 (src/math/utils.h:41-45). */
static int roughlyZero(double x) { return fabs(x) <= EPS_DOUBLE; }

size_t srpPortFragmentCount = 0;   /* fragments that passed coverage + scissor */
size_t srpPortClipOverflow = 0;    /* clipped polygons with more than 6 vertices */

static void message(SRPMessageType type, SRPMessageSeverity sev, const char* fn, const char* fmt, ...)
{
	/* src/utils/message_callback.c:18-35 */
	if (!srpContext.messageCallback.func) return;
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	srpContext.messageCallback.func(type, sev, fn, buf, srpContext.messageCallback.userParameter);
}

static void* xmalloc(size_t n)
{
	/* src/memory/alloc.c:15-22: abort on out-of-memory */
	void* p = malloc(n ? n : 1);
	if (!p) { fprintf(stderr, "srp oracle: out of memory\n"); abort(); }
	return p;
}

/* Per-draw scratch: a chain of blocks released at the end of the draw. */
typedef struct Scratch { struct Scratch* next; size_t used, cap; unsigned char data[]; } Scratch;
static Scratch* scratchHead = NULL;

static void* scratchAlloc(size_t n)
{
	n = (n + 15) & ~(size_t) 15;
	if (!scratchHead || scratchHead->used + n > scratchHead->cap) {
		size_t cap = n > (1u << 20) ? n : (1u << 20);
		Scratch* s = (Scratch*) xmalloc(sizeof(Scratch) + cap);
		s->next = scratchHead; s->used = 0; s->cap = cap;
		scratchHead = s;
	}
	void* p = scratchHead->data + scratchHead->used;
	scratchHead->used += n;
	return p;
}

static void scratchReset(void)
{
	while (scratchHead) { Scratch* n = scratchHead->next; free(scratchHead); scratchHead = n; }
}

/* ---------------------------------------------------------------- context */

void srpNewContext(SRPContext* c)
{
	/* src/core/context.c:15-51 */
	c->messageCallback.func = NULL;
	c->messageCallback.userParameter = NULL;
	c->provokingVertexMode = SRP_PROVOKING_VERTEX_LAST;
	c->raster.frontFace = SRP_WINDING_CCW;
	c->raster.cullFace = SRP_FACE_NONE;
	c->raster.polygonMode = SRP_POLYGON_MODE_FILL;
	c->raster.pointSize = 1.f;
	memset(&c->scissor, 0, sizeof c->scissor);
	c->depth.testEnable = false;
	c->depth.writeEnable = true;
	c->depth.compareOp = SRP_COMPARE_GREATER;
	SRPStencilFaceState f = { SRP_COMPARE_ALWAYS, 0, 0xFF, 0xFF, SRP_STENCIL_KEEP, SRP_STENCIL_KEEP, SRP_STENCIL_KEEP };
	c->stencil.enabled = false;
	c->stencil.front = f;
	c->stencil.back = f;
	c->arena = NULL;
}

/* src/core/context.c:53-180 */
void srpSetMessageCallback(SRPMessageCallback cb) { srpContext.messageCallback = cb; }
void srpProvokingVertexMode(SRPProvokingVertexMode m) { srpContext.provokingVertexMode = m; }
void srpRasterCullFace(SRPFace f) { srpContext.raster.cullFace = f; }
void srpRasterFrontFace(SRPWinding w) { srpContext.raster.frontFace = w; }
void srpRasterPolygonMode(SRPPolygonMode m) { srpContext.raster.polygonMode = m; }
void srpRasterPointSize(float s) { srpContext.raster.pointSize = s; }
void srpScissorTest(bool e) { srpContext.scissor.enabled = e; }
void srpScissorOptions(size_t x, size_t y, size_t w, size_t h)
{
	srpContext.scissor.x = x; srpContext.scissor.y = y;
	srpContext.scissor.width = w; srpContext.scissor.height = h;
}
/* The reference enables the stencil test whatever the argument (context.c:96-99). */
void srpStencilTest(bool e) { (void) e; srpContext.stencil.enabled = true; }
void srpStencilFunc(SRPCompareOp func, uint8_t ref, uint8_t mask)
{
	SRPStencilFaceState* s[2] = { &srpContext.stencil.front, &srpContext.stencil.back };
	for (int i = 0; i < 2; ++i) { s[i]->func = func; s[i]->ref = ref; s[i]->mask = mask; }
}
static SRPStencilFaceState* faceState(SRPFace face)
{
	return face == SRP_FACE_FRONT ? &srpContext.stencil.front : &srpContext.stencil.back;
}
/* FRONT_AND_BACK sets both faces, then falls through to also write the back
 * face again (context.c:116-122); harmless but kept. */
void srpStencilFuncSeparate(SRPFace face, SRPCompareOp func, uint8_t ref, uint8_t mask)
{
	if (face == SRP_FACE_NONE) return;
	if (face == SRP_FACE_FRONT_AND_BACK) srpStencilFunc(func, ref, mask);
	SRPStencilFaceState* s = faceState(face);
	s->func = func; s->ref = ref; s->mask = mask;
}
void srpStencilOp(SRPStencilOp sfail, SRPStencilOp dfail, SRPStencilOp pass)
{
	SRPStencilFaceState* s[2] = { &srpContext.stencil.front, &srpContext.stencil.back };
	for (int i = 0; i < 2; ++i) { s[i]->sfailOp = sfail; s[i]->dfailOp = dfail; s[i]->passOp = pass; }
}
void srpStencilOpSeparate(SRPFace face, SRPStencilOp sfail, SRPStencilOp dfail, SRPStencilOp pass)
{
	if (face == SRP_FACE_NONE) return;
	if (face == SRP_FACE_FRONT_AND_BACK) srpStencilOp(sfail, dfail, pass);
	SRPStencilFaceState* s = faceState(face);
	s->sfailOp = sfail; s->dfailOp = dfail; s->passOp = pass;
}
void srpStencilWriteMask(uint8_t mask)
{
	srpContext.stencil.front.writeMask = mask;
	srpContext.stencil.back.writeMask = mask;
}
void srpStencilWriteMaskSeparate(SRPFace face, uint8_t mask)
{
	if (face == SRP_FACE_NONE) return;
	if (face == SRP_FACE_FRONT_AND_BACK) srpStencilWriteMask(mask);
	faceState(face)->writeMask = mask;
}
void srpDepthTest(bool e) { srpContext.depth.testEnable = e; }
void srpDepthWrite(bool e) { srpContext.depth.writeEnable = e; }
void srpDepthCompareOp(SRPCompareOp op) { srpContext.depth.compareOp = op; }

/* ---------------------------------------------------------------- buffers */

struct SRPVertexBuffer { size_t stride, nVertices, cap; unsigned char* data; };
struct SRPIndexBuffer { SRPType type; size_t elemSize, nIndices, cap; unsigned char* data; };

/* srpSizeofType (src/utils/type.c:15-40): only the unsigned integer types,
 * float and double have a size; anything else is reported and yields 0. */
static size_t indexTypeSize(SRPType t)
{
	switch (t) {
	case SRP_UINT8: return 1;
	case SRP_UINT16: return 2;
	case SRP_UINT32: case SRP_FLOAT: return 4;
	case SRP_UINT64: case SRP_DOUBLE: return 8;
	default:
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpSizeofType", "Unknown type (%i)", t);
		return 0;
	}
}

/* sizeof() of a varying element type (interpolation.c:63-91). */
static size_t typeSize(SRPType t)
{
	switch (t) {
	case SRP_UINT8: case SRP_INT8: return 1;
	case SRP_UINT16: case SRP_INT16: return 2;
	case SRP_UINT32: case SRP_INT32: case SRP_FLOAT: return 4;
	case SRP_UINT64: case SRP_INT64: case SRP_DOUBLE: return 8;
	}
	return 0;
}

SRPVertexBuffer* srpNewVertexBuffer(void)
{
	SRPVertexBuffer* b = (SRPVertexBuffer*) xmalloc(sizeof *b);
	memset(b, 0, sizeof *b);
	return b;
}
void srpFreeVertexBuffer(SRPVertexBuffer* b) { if (b) { free(b->data); free(b); } }
void srpVertexBufferCopyData(SRPVertexBuffer* b, size_t stride, size_t nBytes, const void* data)
{
	/* src/core/buffer.c:30-45 */
	if (nBytes > b->cap) { free(b->data); b->data = (unsigned char*) xmalloc(nBytes); b->cap = nBytes; }
	b->stride = stride;
	b->nVertices = nBytes / stride;
	memcpy(b->data, data, nBytes);
}

SRPIndexBuffer* srpNewIndexBuffer(void)
{
	SRPIndexBuffer* b = (SRPIndexBuffer*) xmalloc(sizeof *b);
	memset(b, 0, sizeof *b);
	b->type = SRP_UINT8;
	b->elemSize = 1;
	return b;
}
void srpFreeIndexBuffer(SRPIndexBuffer* b) { if (b) { free(b->data); free(b); } }
void srpIndexBufferCopyData(SRPIndexBuffer* b, SRPType type, size_t nBytes, const void* data)
{
	/* src/core/buffer.c:77-94 */
	if (nBytes > b->cap) { free(b->data); b->data = (unsigned char*) xmalloc(nBytes); b->cap = nBytes; }
	b->type = type;
	b->elemSize = indexTypeSize(type);
	/* the reference divides by zero here for a type without a size */
	b->nIndices = b->elemSize ? nBytes / b->elemSize : 0;
	memcpy(b->data, data, nBytes);
}

static uint64_t fetchIndex(const SRPIndexBuffer* b, size_t i)
{
	/* src/core/buffer.c:102-128 */
	const unsigned char* p = b->data + i * b->elemSize;
	switch (b->type) {
	case SRP_UINT8: return *p;
	case SRP_UINT16: { uint16_t v; memcpy(&v, p, 2); return v; }
	case SRP_UINT32: { uint32_t v; memcpy(&v, p, 4); return v; }
	case SRP_UINT64: { uint64_t v; memcpy(&v, p, 8); return v; }
	default:
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "indexIndexBuffer", "Unexpected type (%i)", b->type);
		return 0;
	}
}

/* ------------------------------------------------------------ framebuffer */

SRPFramebuffer* srpNewFramebuffer(size_t w, size_t h)
{
	/* src/core/framebuffer.c:17-27 (the reference leaves stencil uninitialised;
	 * the oracle zeroes it so that runs are reproducible) */
	SRPFramebuffer* fb = (SRPFramebuffer*) xmalloc(sizeof *fb);
	fb->width = w; fb->height = h; fb->size = w * h;
	fb->color = (uint32_t*) xmalloc(4 * fb->size);
	fb->depth = (float*) xmalloc(4 * fb->size);
	fb->stencil = (uint8_t*) calloc(fb->size ? fb->size : 1, 1);
	return fb;
}
void srpFreeFramebuffer(SRPFramebuffer* fb) { if (fb) { free(fb->color); free(fb->depth); free(fb->stencil); free(fb); } }
void srpFramebufferClear(const SRPFramebuffer* fb)
{
	/* src/core/framebuffer.c:57-62: colour 0, depth -1, stencil untouched */
	memset(fb->color, 0, 4 * fb->size);
	for (size_t i = 0; i < fb->size; ++i) fb->depth[i] = -1.f;
}

/* NDC -> screen space with the reference's double arithmetic
 * (src/core/framebuffer.c:48-55). */
static void ndcToScreen(const SRPFramebuffer* fb, const float* ndc, float* ss)
{
	ss[0] = (float) (((double) (float) fb->width / 2.) * ((double) ndc[0] + 1.));
	ss[1] = (float) (((double) (float) fb->height / 2.) * (1. - (double) ndc[1]));
	ss[2] = ndc[2];
}

/* ---------------------------------------------------------------- texture */

struct SRPTexture {
	uint8_t* data; int width, height, wm1, hm1; SRPTextureWrappingMode wx, wy;
	/* filtering (an addition: the reference samples the nearest texel only) */
	int filter, nLevels;
	int lw[32], lh[32];
	size_t loff[32];      /* texel offset of each level in mips (levels 1..) */
	uint8_t* mips;
};

SRPTexture* srpNewTextureFromMemory(const uint8_t* texels, int w, int h, int ch,
                                    SRPTextureWrappingMode wx, SRPTextureWrappingMode wy)
{
	if (!texels || w <= 0 || h <= 0 || (ch != 3 && ch != 4)) {
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpNewTextureFromMemory", "Invalid texture arguments");
		return NULL;
	}
	SRPTexture* t = (SRPTexture*) xmalloc(sizeof *t);
	t->data = (uint8_t*) xmalloc((size_t) w * h * 3);
	for (size_t i = 0; i < (size_t) w * h; ++i)
		memcpy(t->data + 3 * i, texels + (size_t) ch * i, 3);
	t->width = w; t->height = h; t->wm1 = w - 1; t->hm1 = h - 1; t->wx = wx; t->wy = wy;
	t->filter = SRP_TEXTURE_FILTER_NEAREST;
	t->nLevels = 1;
	t->lw[0] = w; t->lh[0] = h; t->loff[0] = 0;
	t->mips = NULL;
	return t;
}

SRPTexture* srpNewTexture(const char* path, SRPTextureWrappingMode wx, SRPTextureWrappingMode wy)
{
	/* src/core/texture.c:21-42 */
	SRPImage img;
	const char* err = "";
	if (!srpImageLoad(path, &img, &err)) {
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpNewTexture", "Failed to load image `%s`: %s", path, err);
		return NULL;
	}
	SRPTexture* t = srpNewTextureFromMemory(img.rgb, img.width, img.height, 3, wx, wy);
	free(img.rgb);
	return t;
}

void srpFreeTexture(SRPTexture* t) { if (t) { free(t->data); free(t->mips); free(t); } }

void srpTextureGetFilteredColorLod(const SRPTexture* t, float u, float v, float lod, float out[4]);

void srpTextureGetFilteredColor(const SRPTexture* t, float u, float v, float out[4])
{
	/* src/core/texture.c:56-81: wrap only outside [0, 1], nearest texel,
	 * rows stored top first, alpha 1 (3 stored channels); a texture set to a
	 * filter (an addition) samples level 0 with it. */
	if (t->filter != SRP_TEXTURE_FILTER_NEAREST) { srpTextureGetFilteredColorLod(t, u, v, 0.0f, out); return; }
	if (u < 0 || u > 1) u = (float) (t->wx == TW_REPEAT ? (double) u - floor(u) : fmax(0.0, fmin(1.0, u)));
	if (v < 0 || v > 1) v = (float) (t->wy == TW_REPEAT ? (double) v - floor(v) : fmax(0.0, fmin(1.0, v)));
	float x = (float) t->wm1 * u;
	float y = (float) t->hm1 * (1 - v);
	size_t xi = (size_t) ((double) x + 0.5);
	size_t yi = (size_t) ((double) y + 0.5);
	const uint8_t* p = t->data + 3 * (xi + yi * (size_t) t->width);
	const float inv255 = (float) (1. / 255.);
	out[0] = p[0] * inv255;
	out[1] = p[1] * inv255;
	out[2] = p[2] * inv255;
	out[3] = 1.f;
}

/* ------------------------------------------------------ texture filtering
 * Not in the reference (its README.md:71-72 lists bilinear filtering and
 * mipmapping as to do): the definition of srp/texture.h, restated here in
 * plain C as the checker of the device sampler. */

int srpTextureMipLevels(int w, int h)
{
	int n = 1;
	while (w > 1 || h > 1) { w = w > 1 ? w / 2 : 1; h = h > 1 ? h / 2 : 1; ++n; }
	return n;
}

static const uint8_t* texel(const SRPTexture* t, int l, int x, int y)
{
	if (l == 0) return t->data + 3 * ((size_t) y * t->width + x);
	return t->mips + 3 * (t->loff[l] + (size_t) y * t->lw[l] + x);
}

static void buildMips(SRPTexture* t)
{
	const int n = srpTextureMipLevels(t->width, t->height);
	size_t total = 0;
	int w = t->width, h = t->height;
	for (int l = 1; l < n; ++l) {
		w = w > 1 ? w / 2 : 1; h = h > 1 ? h / 2 : 1;
		t->lw[l] = w; t->lh[l] = h; t->loff[l] = total;
		total += (size_t) w * h;
	}
	t->mips = (uint8_t*) xmalloc(total * 3 + 3);
	for (int l = 1; l < n; ++l) {
		const int pw = t->lw[l - 1], ph = t->lh[l - 1];
		for (int j = 0; j < t->lh[l]; ++j)
			for (int i = 0; i < t->lw[l]; ++i) {
				const int x0 = 2 * i < pw ? 2 * i : pw - 1, x1 = 2 * i + 1 < pw ? 2 * i + 1 : pw - 1;
				const int y0 = 2 * j < ph ? 2 * j : ph - 1, y1 = 2 * j + 1 < ph ? 2 * j + 1 : ph - 1;
				const uint8_t *a = texel(t, l - 1, x0, y0), *b = texel(t, l - 1, x1, y0);
				const uint8_t *c = texel(t, l - 1, x0, y1), *d = texel(t, l - 1, x1, y1);
				uint8_t* o = t->mips + 3 * (t->loff[l] + (size_t) j * t->lw[l] + i);
				for (int k = 0; k < 3; ++k) o[k] = (uint8_t) ((a[k] + b[k] + c[k] + d[k] + 2) / 4);
			}
	}
	t->nLevels = n;
}

void srpTextureSetFilter(SRPTexture* t, SRPTextureFilter f)
{
	if (f != SRP_TEXTURE_FILTER_NEAREST && f != SRP_TEXTURE_FILTER_BILINEAR && f != SRP_TEXTURE_FILTER_TRILINEAR) {
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpTextureSetFilter",
		        "Unknown texture filter (%i). Falling back to SRP_TEXTURE_FILTER_NEAREST", (int) f);
		f = SRP_TEXTURE_FILTER_NEAREST;
	}
	t->filter = f;
	if (f == SRP_TEXTURE_FILTER_TRILINEAR && !t->mips) buildMips(t);
}

SRPTextureFilter srpTextureGetFilter(const SRPTexture* t) { return (SRPTextureFilter) t->filter; }

/* Bilinear sample of level l at wrapped (u, v), channels in 0..255. */
static void bilinear(const SRPTexture* t, int l, float u, float v, float c[3])
{
	const int w = t->lw[l], h = t->lh[l];
	const float x = (float) (w - 1) * u, y = (float) (h - 1) * (1.0f - v);
	const float fx0 = floorf(x), fy0 = floorf(y);
	int x0 = (int) fx0, y0 = (int) fy0;
	if (x0 < 0) x0 = 0;
	if (x0 > w - 1) x0 = w - 1;
	if (y0 < 0) y0 = 0;
	if (y0 > h - 1) y0 = h - 1;
	const float fx = x - fx0, fy = y - fy0;
	const int x1 = x0 + 1 < w ? x0 + 1 : (t->wx == TW_REPEAT ? 0 : w - 1);
	const int y1 = y0 + 1 < h ? y0 + 1 : (t->wy == TW_REPEAT ? 0 : h - 1);
	const uint8_t *a = texel(t, l, x0, y0), *b = texel(t, l, x1, y0), *d = texel(t, l, x0, y1), *e = texel(t, l, x1, y1);
	for (int k = 0; k < 3; ++k) {
		const float top = (float) a[k] + fx * ((float) b[k] - (float) a[k]);
		const float bot = (float) d[k] + fx * ((float) e[k] - (float) d[k]);
		c[k] = top + fy * (bot - top);
	}
}

void srpTextureGetFilteredColorLod(const SRPTexture* t, float u, float v, float lod, float out[4])
{
	if (t->filter == SRP_TEXTURE_FILTER_NEAREST) { srpTextureGetFilteredColor(t, u, v, out); return; }
	if (u < 0 || u > 1) u = (float) (t->wx == TW_REPEAT ? (double) u - floor(u) : fmax(0.0, fmin(1.0, u)));
	if (v < 0 || v > 1) v = (float) (t->wy == TW_REPEAT ? (double) v - floor(v) : fmax(0.0, fmin(1.0, v)));
	float c[3];
	bilinear(t, 0, u, v, c);
	if (t->filter == SRP_TEXTURE_FILTER_TRILINEAR && t->nLevels > 1) {
		const float top = (float) (t->nLevels - 1);
		const float ld = lod > 0.0f ? (lod < top ? lod : top) : 0.0f;
		const int l0 = (int) floorf(ld);
		const float f = ld - (float) l0;
		float c0[3], c1[3];
		bilinear(t, l0, u, v, c0);
		bilinear(t, l0 + 1 < t->nLevels ? l0 + 1 : l0, u, v, c1);
		for (int k = 0; k < 3; ++k) c[k] = c0[k] + f * (c1[k] - c0[k]);
	}
	const float inv255 = (float) (1. / 255.);
	for (int k = 0; k < 3; ++k) out[k] = c[k] * inv255;
	out[3] = 1.f;
}

int srpTextureGet(SRPTexture* t, SRPTextureParameter p)
{
	switch (p) {
	case SRP_TEXTURE_WRAPPING_MODE_X: return t->wx;
	case SRP_TEXTURE_WRAPPING_MODE_Y: return t->wy;
	}
	message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpTextureGet", "Unknown texture parameter (%i)", p);
	return -1;
}

void srpTextureSet(SRPTexture* t, SRPTextureParameter p, int data)
{
	/* src/core/texture.c:102-137 (stores the value even when it is invalid) */
	if (p != SRP_TEXTURE_WRAPPING_MODE_X && p != SRP_TEXTURE_WRAPPING_MODE_Y) {
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpTextureSet", "Unknown texture parameter (%i)", p);
		return;
	}
	if (p == SRP_TEXTURE_WRAPPING_MODE_X) t->wx = (SRPTextureWrappingMode) data;
	else t->wy = (SRPTextureWrappingMode) data;
	if (data != TW_REPEAT && data != TW_CLAMP_TO_EDGE)
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "srpTextureSet",
		        "Unknown texture wrapping mode (%i). Falling back to TW_REPEAT", data);
}

/* ---------------------------------------------------------- interpolation */

/* Weighted sum of the varyings of n vertices into `out`
 * (src/pipeline/interpolation.c:63-163). invW == NULL means clip-time
 * interpolation, which is affine for every floating varying. Integer varyings
 * are always copied from the provoking vertex. */
static void interpolateVaryings(const SRPVertexShaderOut* v, size_t n, const float* w,
                                const float* invW, float recip, const SRPShaderProgram* sp, void* out)
{
	const size_t prov = srpContext.provokingVertexMode == SRP_PROVOKING_VERTEX_FIRST ? 0 : n - 1;
	size_t off = 0;
	for (size_t a = 0; a < sp->vs->nVaryings; ++a) {
		const SRPVaryingInfo* info = &sp->vs->varyingsInfo[a];
		int persp = info->interpolationMode == SRP_INTERPOLATION_MODE_PERSPECTIVE;
		int affine = info->interpolationMode == SRP_INTERPOLATION_MODE_AFFINE;
		if (!invW) { persp = 0; affine = 1; }
		size_t es = typeSize(info->type);
		unsigned char* dst = (unsigned char*) out + off;
		if (info->type == SRP_FLOAT) {
			for (size_t e = 0; e < info->nItems; ++e) {
				float val = 0.;
				if (persp) {
					for (size_t i = 0; i < n; ++i) {
						float x; memcpy(&x, (const unsigned char*) v[i].varyings + off + 4 * e, 4);
						val += x * invW[i] * w[i];
					}
					val *= recip;
				} else if (affine) {
					for (size_t i = 0; i < n; ++i) {
						float x; memcpy(&x, (const unsigned char*) v[i].varyings + off + 4 * e, 4);
						val += x * w[i];
					}
				} else
					memcpy(&val, (const unsigned char*) v[prov].varyings + off + 4 * e, 4);
				memcpy(dst + 4 * e, &val, 4);
			}
		} else if (info->type == SRP_DOUBLE) {
			for (size_t e = 0; e < info->nItems; ++e) {
				double val = 0.;
				if (persp) {
					for (size_t i = 0; i < n; ++i) {
						double x; memcpy(&x, (const unsigned char*) v[i].varyings + off + 8 * e, 8);
						val += x * invW[i] * w[i];
					}
					val *= recip;
				} else if (affine) {
					for (size_t i = 0; i < n; ++i) {
						double x; memcpy(&x, (const unsigned char*) v[i].varyings + off + 8 * e, 8);
						val += x * w[i];
					}
				} else
					memcpy(&val, (const unsigned char*) v[prov].varyings + off + 8 * e, 8);
				memcpy(dst + 8 * e, &val, 8);
			}
		} else if (es) {
			memcpy(dst, (const unsigned char*) v[prov].varyings + off, es * info->nItems);
		} else {
			message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "interpolateAttributes", "Unexpected type (%i)", info->type);
		}
		off += es * info->nItems;
	}
}

/* -------------------------------------------------------- vertex handling */

typedef struct VCache { size_t base, size; unsigned char* valid; SRPVertexShaderOut* out; unsigned char* vary; } VCache;

static void runVertexShader(size_t vi, unsigned char* varyDst, const SRPVertexBuffer* vb,
                            const SRPShaderProgram* sp, SRPVertexShaderOut* out)
{
	/* src/pipeline/vertex_processing.c:55-74 */
	SRPVertexShaderIn in;
	in.uniform = sp->uniform;
	in.vertex = (SRPVertex*) (vb->data + vi * vb->stride);
	in.vertexID = vi;
	memset(out->clipPosition, 0, sizeof out->clipPosition);
	out->varyings = (SRPVarying*) varyDst;
	sp->vs->shader(&in, out);
}

static void cacheInit(VCache* c, const SRPIndexBuffer* ib, size_t start, size_t count, size_t varySize)
{
	/* src/pipeline/vertex_processing.c:23-36 and :90-112 (min/max over the
	 * referenced vertices, one slot per vertex in between) */
	size_t lo = SIZE_MAX, hi = 0;
	if (ib) {
		for (size_t i = 0; i < count; ++i) {
			size_t vi = (size_t) fetchIndex(ib, start + i);
			if (vi < lo) lo = vi;
			if (vi > hi) hi = vi;
		}
	} else { lo = start; hi = start + count - 1; }
	c->base = lo;
	c->size = hi - lo + 1;
	c->valid = (unsigned char*) scratchAlloc(c->size);
	memset(c->valid, 0, c->size);
	c->out = (SRPVertexShaderOut*) scratchAlloc(sizeof(SRPVertexShaderOut) * c->size);
	c->vary = (unsigned char*) scratchAlloc(varySize * c->size + 1);
}

static SRPVertexShaderOut* cacheFetch(VCache* c, size_t vi, const SRPVertexBuffer* vb, const SRPShaderProgram* sp)
{
	/* src/pipeline/vertex_processing.c:38-53 */
	size_t k = vi - c->base;
	if (!c->valid[k]) {
		runVertexShader(vi, c->vary + k * sp->vs->varyingsSize, vb, sp, &c->out[k]);
		c->valid[k] = 1;
	}
	return &c->out[k];
}

/* invW = (float)(1.0 / (double) w); xyz *= invW; w = 1
 * (src/pipeline/vertex_processing.c:76-88). */
static void perspectiveDivide(SRPVertexShaderOut* v, float* invWOut)
{
	float invW = (float) (1.0 / (double) v->clipPosition[3]);
	if (invWOut) *invWOut = invW;
	v->ndcPosition[0] *= invW;
	v->ndcPosition[1] *= invW;
	v->ndcPosition[2] *= invW;
	v->ndcPosition[3] = 1.f;
}

/* --------------------------------------------------------------- clipping */

static float planeDist(const SRPVertexShaderOut* v, int p)
{
	/* src/pipeline/clipping.c:260-277 */
	const float* c = v->clipPosition;
	switch (p) {
	case 0: return c[0] + c[3];
	case 1: return c[3] - c[0];
	case 2: return c[1] + c[3];
	case 3: return c[3] - c[1];
	case 4: return c[2] + c[3];
	default: return c[3] - c[2];
	}
}

static unsigned outcode(const SRPVertexShaderOut* v)
{
	/* src/pipeline/clipping.c:121-137 */
	const float* c = v->clipPosition;
	unsigned code = 0;
	code |= (unsigned) (c[0] + c[3] < 0) << 0;
	code |= (unsigned) (c[3] - c[0] < 0) << 1;
	code |= (unsigned) (c[1] + c[3] < 0) << 2;
	code |= (unsigned) (c[3] - c[1] < 0) << 3;
	code |= (unsigned) (c[2] + c[3] < 0) << 4;
	code |= (unsigned) (c[3] - c[2] < 0) << 5;
	return code;
}

/* New vertex a*(1-t) + b*t, varyings interpolated affinely
 * (src/pipeline/clipping.c:244-258). */
static void lerpVertex(const SRPVertexShaderOut* a, const SRPVertexShaderOut* b, float t,
                       const SRPShaderProgram* sp, SRPVertexShaderOut* out)
{
	for (int i = 0; i < 4; ++i)
		out->clipPosition[i] = a->clipPosition[i] * (1 - t) + b->clipPosition[i] * t;
	void* vary = scratchAlloc(sp->vs->varyingsSize + 1);
	SRPVertexShaderOut pair[2] = { *a, *b };
	const float w[2] = { 1 - t, t };
	interpolateVaryings(pair, 2, w, NULL, 0.f, sp, vary);
	out->varyings = (SRPVarying*) vary;
}

#define MAX_POLY 16

/* One Sutherland-Hodgman pass (src/pipeline/clipping.c:199-242). */
static size_t clipPlane(const SRPVertexShaderOut* in, size_t n, int plane, const SRPShaderProgram* sp,
                        SRPVertexShaderOut* out)
{
	size_t m = 0;
	for (size_t i = 0; i < n; ++i) {
		const SRPVertexShaderOut* cur = &in[i];
		const SRPVertexShaderOut* nxt = &in[(i + 1) % n];
		float da = planeDist(cur, plane), db = planeDist(nxt, plane);
		int cin = da >= 0, nin = db >= 0;
		if (cin && nin) out[m++] = *nxt;
		else if (cin || nin) {
			if (roughlyZero(da - db)) continue;
			float t = da / (da - db);
			lerpVertex(cur, nxt, t, sp, &out[m++]);
			if (!cin && nin) out[m++] = *nxt;
		}
		if (m > MAX_POLY - 2) break;
	}
	return m;
}

/* Trivial accept/reject, then the six planes L,R,B,T,N,F, then a fan
 * (src/pipeline/clipping.c:68-119). Returns the number of triangles. */
static size_t clipTri(const SRPVertexShaderOut in[3], const SRPShaderProgram* sp, SRPVertexShaderOut out[][3])
{
	unsigned c0 = outcode(&in[0]), c1 = outcode(&in[1]), c2 = outcode(&in[2]);
	if ((c0 | c1 | c2) == 0) { out[0][0] = in[0]; out[0][1] = in[1]; out[0][2] = in[2]; return 1; }
	if (c0 & c1 & c2) return 0;
	SRPVertexShaderOut A[MAX_POLY], B[MAX_POLY];
	SRPVertexShaderOut *src = A, *dst = B;
	size_t n = 3;
	for (int i = 0; i < 3; ++i) src[i] = in[i];
	for (int p = 0; p < 6; ++p) {
		n = clipPlane(src, n, p, sp, dst);
		if (n == 0) return 0;
		SRPVertexShaderOut* t = src; src = dst; dst = t;
	}
	if (n > 6) ++srpPortClipOverflow;  /* the reference overflows its 6-entry buffers here */
	size_t k = 0;
	for (size_t i = 1; i + 1 < n; ++i, ++k) { out[k][0] = src[0]; out[k][1] = src[i]; out[k][2] = src[i + 1]; }
	return k;
}

/* Liang-Barsky style parametric clip (src/pipeline/clipping.c:139-183).
 * Returns 1 when the line is rejected. */
static int clipLineSeg(SRPVertexShaderOut v[2], const SRPShaderProgram* sp)
{
	unsigned c0 = outcode(&v[0]), c1 = outcode(&v[1]);
	if ((c0 | c1) == 0) return 0;
	if (c0 & c1) return 1;
	float t0 = 0.f, t1 = 1.f;
	for (int p = 0; p < 6; ++p) {
		float da = planeDist(&v[0], p), db = planeDist(&v[1], p);
		if (da < 0. && db < 0.) return 1;
		if (da < 0. || db < 0.) {
			if (roughlyZero(da - db)) continue;
			float t = da / (da - db);
			if (da < 0.) t0 = t0 > t ? t0 : t;
			else t1 = t1 > t ? t : t1;
			if (t0 > t1) return 1;
		}
	}
	SRPVertexShaderOut a = v[0], b = v[1];
	if (t0 > 0.) lerpVertex(&a, &b, t0, sp, &v[0]);
	if (t1 < 1.) lerpVertex(&a, &b, t1, sp, &v[1]);
	return 0;
}

/* Whole-point reject (src/pipeline/clipping.c:185-197). */
static int clipPointV(const SRPVertexShaderOut* v)
{
	float x = v->clipPosition[0], y = v->clipPosition[1], z = v->clipPosition[2], w = v->clipPosition[3];
	return (x < -w || x > w) || (y < -w || y > w) || (z < -w || z > w);
}

/* ------------------------------------------------------- fragment stage */

static int scissorPass(size_t x, size_t y)
{
	/* src/raster/fragment.c:127-140 */
	if (!srpContext.scissor.enabled) return 1;
	size_t x0 = srpContext.scissor.x, x1 = x0 + srpContext.scissor.width;
	size_t y0 = srpContext.scissor.y, y1 = y0 + srpContext.scissor.height;
	return !(x < x0 || x >= x1 || y < y0 || y >= y1);
}

static int cmpStencil(uint8_t ref, uint8_t stored, uint8_t mask, SRPCompareOp op)
{
	/* src/raster/fragment.c:156-178 */
	uint8_t l = ref & mask, r = stored & mask;
	switch (op) {
	case SRP_COMPARE_NEVER: return 0;
	case SRP_COMPARE_ALWAYS: return 1;
	case SRP_COMPARE_LESS: return l < r;
	case SRP_COMPARE_LEQUAL: return l <= r;
	case SRP_COMPARE_GREATER: return l > r;
	case SRP_COMPARE_GEQUAL: return l >= r;
	case SRP_COMPARE_EQUAL: return l == r;
	case SRP_COMPARE_NOTEQUAL: return l != r;
	}
	message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "stencilCompare",
	        "Unknown stencil operation (%i), fallback to SRP_COMPARE_NEVER", op);
	return 0;
}

static uint8_t stencilOpValue(SRPStencilOp op, uint8_t s, uint8_t ref)
{
	/* src/raster/fragment.c:204-223 */
	switch (op) {
	case SRP_STENCIL_KEEP: return s;
	case SRP_STENCIL_ZERO: return 0;
	case SRP_STENCIL_REPLACE: return ref;
	case SRP_STENCIL_INCR: return s < 255 ? s + 1 : 255;
	case SRP_STENCIL_INCR_WRAP: return (uint8_t) (s + 1);
	case SRP_STENCIL_DECR: return s > 0 ? s - 1 : 0;
	case SRP_STENCIL_DECR_WRAP: return (uint8_t) (s - 1);
	case SRP_STENCIL_INVERT: return (uint8_t) ~s;
	}
	message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "applyStencilOp",
	        "Unknown stencil operation (%i), fallback to SRP_STENCIL_KEEP", op);
	return s;
}

static void stencilUpdate(uint8_t* s, const SRPStencilFaceState* st, SRPStencilOp op)
{
	/* src/raster/fragment.c:180-202: only the write-mask bits change */
	uint8_t cur = *s;
	uint8_t val = stencilOpValue(op, *s, st->ref);
	*s = (uint8_t) ((cur & ~st->writeMask) | (val & st->writeMask));
}

static int depthPass(float in, float stored)
{
	/* src/raster/fragment.c:225-245 */
	if (!srpContext.depth.testEnable) return 1;
	switch (srpContext.depth.compareOp) {
	case SRP_COMPARE_NEVER: return 0;
	case SRP_COMPARE_ALWAYS: return 1;
	case SRP_COMPARE_LESS: return in < stored;
	case SRP_COMPARE_LEQUAL: return in <= stored;
	case SRP_COMPARE_GREATER: return in > stored;
	case SRP_COMPARE_GEQUAL: return in >= stored;
	case SRP_COMPARE_EQUAL: return in == stored;
	case SRP_COMPARE_NOTEQUAL: return in != stored;
	}
	return 0;
}

static uint32_t packColor(const float c[4])
{
	/* src/core/color.c:14-23: clamp(c * 255) truncated to 8 bits, packed R<<24|G<<16|B<<8|A */
	uint32_t r = 0;
	for (int k = 0; k < 4; ++k) {
		float v = c[k] * 255;
		float cl = (v < 0) ? 0.f : (v > 255) ? 255.f : v;
		r = (r << 8) | (uint8_t) cl;
	}
	return r;
}

/* Scissor, stencil, early or late depth, shader, stencil pass op, colour and
 * depth write (src/raster/fragment.c:63-125). */
static void fragment(const SRPFramebuffer* fb, const SRPShaderProgram* sp, int x, int y, SRPFragmentShaderIn* in)
{
	if (!scissorPass((size_t) x, (size_t) y)) return;
	++srpPortFragmentCount;
	/* The pixel index is y * width + x; a line end at x == width lands on the
	 * next row exactly as in the reference. Indices past the end of the
	 * buffer (undefined behaviour in the reference) are dropped. */
	size_t idx = (size_t) y * fb->width + (size_t) x;
	if (idx >= fb->size) return;
	uint32_t* pc = &fb->color[idx];
	float* pd = &fb->depth[idx];
	uint8_t* ps = &fb->stencil[idx];
	const int early = !sp->fs->mayOverwriteDepth;
	const int sten = srpContext.stencil.enabled;
	const SRPStencilFaceState* st = in->frontFacing ? &srpContext.stencil.front : &srpContext.stencil.back;
	const float stored = *pd;
	float depth = in->fragCoord[2];
	if (sten && !cmpStencil(st->ref, *ps, st->mask, st->func)) { stencilUpdate(ps, st, st->sfailOp); return; }
	if (early && !depthPass(depth, stored)) { if (sten) stencilUpdate(ps, st, st->dfailOp); return; }
	SRPFragmentShaderOut out;
	memset(&out, 0, sizeof out);
	out.fragDepth = NAN;
	sp->fs->shader(in, &out);
	if (!early) {
		if (!isnan(out.fragDepth)) depth = out.fragDepth;
		if (!depthPass(depth, stored)) { if (sten) stencilUpdate(ps, st, st->dfailOp); return; }
	}
	if (sten) stencilUpdate(ps, st, st->passOp);
	*pc = packColor(out.color);
	if (srpContext.depth.testEnable && srpContext.depth.writeEnable) *pd = depth;
}

/* --------------------------------------------------------------- triangle */

typedef struct Tri {
	SRPVertexShaderOut v[3];
	float ss[3][3], edge[3][3];
	int tl[3];
	float minx, miny, maxx, maxy;
	float lam[3], lamRow[3], dx[3], dy[3];
	float invW[3];
	int front;
	size_t id;
} Tri;

static float cross2(float ax, float ay, float bx, float by) { return ax * by - ay * bx; }

/* Perspective divide, NDC cull and winding fix, screen-space edges,
 * degenerate reject, bbox, barycentrics at the first pixel centre and the
 * top-left flags (src/raster/triangle.c:113-238). Returns 0 if culled. */
static int setupTri(Tri* t, const SRPFramebuffer* fb)
{
	for (int i = 0; i < 3; ++i) perspectiveDivide(&t->v[i], &t->invW[i]);
	/* signed NDC area of (v1 - v0) x (v2 - v0), triangle.c:162-182 */
	const float* p0 = t->v[0].ndcPosition;
	const float* p1 = t->v[1].ndcPosition;
	const float* p2 = t->v[2].ndcPosition;
	float e0x = p1[0] - p0[0], e0y = p1[1] - p0[1];
	float e1x = p2[0] - p0[0], e1y = p2[1] - p0[1];
	float area = cross2(e0x, e0y, e1x, e1y);
	int ccw = area > 0;
	if (srpContext.raster.cullFace == SRP_FACE_FRONT_AND_BACK) return 0;
	int front = ((area > 0) & (srpContext.raster.frontFace == SRP_WINDING_CCW)) ||
	            ((area < 0) & (srpContext.raster.frontFace == SRP_WINDING_CW));
	int cull = (front && srpContext.raster.cullFace == SRP_FACE_FRONT) ||
	           (!front && srpContext.raster.cullFace == SRP_FACE_BACK);
	t->front = front;
	if (cull) return 0;
	if (!ccw) {
		/* triangle.c:184-195: swap vertices 1 and 2 (and their 1/w) */
		SRPVertexShaderOut tv = t->v[1]; t->v[1] = t->v[2]; t->v[2] = tv;
		float tw = t->invW[1]; t->invW[1] = t->invW[2]; t->invW[2] = tw;
	}
	for (int i = 0; i < 3; ++i) ndcToScreen(fb, t->v[i].ndcPosition, t->ss[i]);
	for (int i = 0; i < 3; ++i)
		for (int k = 0; k < 3; ++k) t->edge[i][k] = t->ss[(i + 1) % 3][k] - t->ss[i][k];
	float areaX2 = fabsf(cross2(t->edge[0][0], t->edge[0][1], t->edge[2][0], t->edge[2][1]));
	if (roughlyZero(areaX2)) return 0;
	/* bbox: floor/ceil in double, clamped to [0, W] x [0, H] (triangle.c:142-149) */
	float mnx = t->ss[0][0], mny = t->ss[0][1], mxx = t->ss[0][0], mxy = t->ss[0][1];
	/* MIN(a, MIN(b, c)) with MIN(p, q) = p > q ? q : p */
	{
		float m;
		m = t->ss[1][0] > t->ss[2][0] ? t->ss[2][0] : t->ss[1][0]; mnx = t->ss[0][0] > m ? m : t->ss[0][0];
		m = t->ss[1][1] > t->ss[2][1] ? t->ss[2][1] : t->ss[1][1]; mny = t->ss[0][1] > m ? m : t->ss[0][1];
		m = t->ss[1][0] > t->ss[2][0] ? t->ss[1][0] : t->ss[2][0]; mxx = t->ss[0][0] > m ? t->ss[0][0] : m;
		m = t->ss[1][1] > t->ss[2][1] ? t->ss[1][1] : t->ss[2][1]; mxy = t->ss[0][1] > m ? t->ss[0][1] : m;
	}
	double fx = floor(mnx), fy = floor(mny), cx = ceil(mxx), cy = ceil(mxy);
	t->minx = (float) (fx > 0 ? fx : 0);
	t->miny = (float) (fy > 0 ? fy : 0);
	t->maxx = (float) (cx > (double) fb->width ? (double) fb->width : cx);
	t->maxy = (float) (cy > (double) fb->height ? (double) fb->height : cy);
	/* barycentrics at the centre of the first pixel (triangle.c:197-226);
	 * lambda[i] pairs with edge (i + 1) % 3 */
	float px = (float) ((double) t->minx + 0.5), py = (float) ((double) t->miny + 0.5);
	float ap[2] = { px - t->ss[0][0], py - t->ss[0][1] };
	float bp[2] = { px - t->ss[1][0], py - t->ss[1][1] };
	float cp[2] = { px - t->ss[2][0], py - t->ss[2][1] };
	t->lam[0] = cross2(bp[0], bp[1], t->edge[1][0], t->edge[1][1]) / areaX2;
	t->lam[1] = cross2(cp[0], cp[1], t->edge[2][0], t->edge[2][1]) / areaX2;
	t->lam[2] = cross2(ap[0], ap[1], t->edge[0][0], t->edge[0][1]) / areaX2;
	t->dx[0] = t->edge[1][1] / areaX2;
	t->dx[1] = t->edge[2][1] / areaX2;
	t->dx[2] = t->edge[0][1] / areaX2;
	t->dy[0] = -t->edge[1][0] / areaX2;
	t->dy[1] = -t->edge[2][0] / areaX2;
	t->dy[2] = -t->edge[0][0] / areaX2;
	for (int i = 0; i < 3; ++i) {
		t->lamRow[i] = t->lam[i];
		/* edge i is "top or left" (triangle.c:235-238), used with lambda[i] */
		t->tl[i] = (t->edge[i][0] > 0 && roughlyZero(t->edge[i][1])) || (t->edge[i][1] < 0);
	}
	return 1;
}

/* Row-major bbox walk with incremental barycentrics and the top-left rule
 * (src/raster/triangle.c:73-111, 240-247; interpolation.c:34-47). */
static void rasterTri(Tri* t, const SRPFramebuffer* fb, const SRPShaderProgram* sp, void* interp)
{
	for (size_t y = (size_t) t->miny; (float) y < t->maxy; ++y) {
		for (size_t x = (size_t) t->minx; (float) x < t->maxx; ++x) {
			int inside = 1;
			for (int i = 0; i < 3; ++i)
				if (!((t->lam[i] > 0.) || (roughlyZero(t->lam[i]) && t->tl[i]))) { inside = 0; break; }
			if (inside) {
				float recip = 1 / (t->invW[0] * t->lam[0] + t->invW[1] * t->lam[1] + t->invW[2] * t->lam[2]);
				float depth = t->v[0].ndcPosition[2] * t->invW[0] * t->lam[0]
				            + t->v[1].ndcPosition[2] * t->invW[1] * t->lam[1]
				            + t->v[2].ndcPosition[2] * t->invW[2] * t->lam[2];
				interpolateVaryings(t->v, 3, t->lam, t->invW, recip, sp, interp);
				SRPFragmentShaderIn in;
				in.uniform = sp->uniform;
				in.varyings = (SRPInterpolated*) interp;
				in.fragCoord[0] = (float) ((double) x + 0.5);
				in.fragCoord[1] = (float) ((double) y + 0.5);
				in.fragCoord[2] = depth;
				in.fragCoord[3] = recip;
				in.frontFacing = t->front;
				in.primitiveID = t->id;
				fragment(fb, sp, (int) x, (int) y, &in);
			}
			for (int i = 0; i < 3; ++i) t->lam[i] += t->dx[i];
		}
		for (int i = 0; i < 3; ++i) { t->lamRow[i] += t->dy[i]; t->lam[i] = t->lamRow[i]; }
	}
}

/* ------------------------------------------------------------------- line */

typedef struct Line { SRPVertexShaderOut v[2]; float ss[2][3]; float invW[2]; size_t id; } Line;

static void setupLn(Line* l, const SRPFramebuffer* fb)
{
	/* src/raster/line.c:79-86 (the reference also divides a third, out-of-range
	 * slot; that write lands in fields recomputed right after and is omitted) */
	for (int i = 0; i < 2; ++i) perspectiveDivide(&l->v[i], &l->invW[i]);
	for (int i = 0; i < 2; ++i) ndcToScreen(fb, l->v[i].ndcPosition, l->ss[i]);
}

/* DDA with steps = ceil(max |dx|, |dy|), fp32 position and parameter
 * accumulators, round-half-away pixel snapping (src/raster/line.c:34-96). */
static void rasterLn(Line* l, const SRPFramebuffer* fb, const SRPShaderProgram* sp, void* interp)
{
	float dx = l->ss[1][0] - l->ss[0][0];
	float dy = l->ss[1][1] - l->ss[0][1];
	int steps = (int) ceil(fmax(fabs(dx), fabs(dy)));
	if (steps == 0) steps = 1;
	float xInc = dx / steps, yInc = dy / steps;
	float tInc = (float) (1. / steps);
	float x = l->ss[0][0], y = l->ss[0][1], t = 0.f;
	for (int i = 0; i <= steps; ++i) {
		int px = (int) round(x), py = (int) round(y);
		const float w[2] = { 1 - t, t };
		float recip = 1 / (l->invW[0] * w[0] + l->invW[1] * w[1]);
		float depth = l->v[0].ndcPosition[2] * l->invW[0] * w[0] + l->v[1].ndcPosition[2] * l->invW[1] * w[1];
		interpolateVaryings(l->v, 2, w, l->invW, recip, sp, interp);
		SRPFragmentShaderIn in;
		in.uniform = sp->uniform;
		in.varyings = (SRPInterpolated*) interp;
		in.fragCoord[0] = (float) ((double) px + 0.5);
		in.fragCoord[1] = (float) ((double) py + 0.5);
		in.fragCoord[2] = depth;
		in.fragCoord[3] = recip;
		in.frontFacing = true;
		in.primitiveID = l->id;
		fragment(fb, sp, px, py, &in);
		x += xInc; y += yInc; t += tInc;
	}
}

/* ------------------------------------------------------------------ point */

typedef struct Point { SRPVertexShaderOut v; size_t id; } Point;

/* Square [ss - size/2, ss + size/2) tested at pixel centres inside the
 * framebuffer-clamped integer bounds (src/raster/point.c:32-118). */
static void rasterPt(Point* p, const SRPFramebuffer* fb, const SRPShaderProgram* sp)
{
	const float size = srpContext.raster.pointSize;
	float ss[3];
	ndcToScreen(fb, p->v.ndcPosition, ss);
	float half = (float) (size * 0.5);
	float mnx = ss[0] - half, mny = ss[1] - half, mxx = ss[0] + half, mxy = ss[1] + half;
	int x0 = (int) floor(mnx), x1 = (int) floor(mxx), y0 = (int) floor(mny), y1 = (int) floor(mxy);
	if (x1 < 0 || y1 < 0 || x0 >= (int) fb->width || y0 >= (int) fb->height) return;
	if (x0 < 0) x0 = 0;
	if (y0 < 0) y0 = 0;
	if (x1 >= (int) fb->width) x1 = (int) fb->width - 1;
	if (y1 >= (int) fb->height) y1 = (int) fb->height - 1;
	for (int y = y0; y <= y1; ++y)
		for (int x = x0; x <= x1; ++x) {
			float cx = (float) (x + 0.5), cy = (float) (y + 0.5);
			if (cx < mnx || cx >= mxx || cy < mny || cy >= mxy) continue;
			SRPFragmentShaderIn in;
			in.uniform = sp->uniform;
			in.varyings = (SRPInterpolated*) p->v.varyings;
			in.fragCoord[0] = cx;
			in.fragCoord[1] = cy;
			in.fragCoord[2] = p->v.ndcPosition[2];
			in.fragCoord[3] = p->v.ndcPosition[3];
			in.frontFacing = true;
			in.primitiveID = p->id;
			fragment(fb, sp, x, y, &in);
		}
}

/* --------------------------------------------------------------- assembly */

static size_t triCount(size_t n, SRPPrimitive p)
{
	/* src/pipeline/topology.c:14-22 */
	if (p == SRP_PRIM_TRIANGLES) return n / 3;
	return n >= 3 ? n - 2 : 0;
}

static void triStream(size_t base, size_t k, SRPPrimitive p, size_t out[3])
{
	/* src/pipeline/topology.c:24-48 */
	if (p == SRP_PRIM_TRIANGLES) { out[0] = base + 3 * k; out[1] = out[0] + 1; out[2] = out[0] + 2; }
	else if (p == SRP_PRIM_TRIANGLE_STRIP) {
		int odd = (int) (k & 1);
		out[0] = base + k + (odd ? 1 : 0);
		out[1] = base + k + (odd ? 0 : 1);
		out[2] = base + k + 2;
	} else { out[0] = base; out[1] = base + k + 1; out[2] = base + k + 2; }
}

static size_t lineCount(size_t n, SRPPrimitive p)
{
	/* src/pipeline/topology.c:50-60 */
	if (p == SRP_PRIM_LINES) return n / 2;
	if (p == SRP_PRIM_LINE_STRIP) return n != 1 ? n - 1 : 0;
	return n != 1 ? n : 0;
}

static void lineStream(size_t base, size_t k, SRPPrimitive p, size_t n, size_t out[2])
{
	/* src/pipeline/topology.c:62-83 */
	if (p == SRP_PRIM_LINES) { out[0] = base + 2 * k; out[1] = out[0] + 1; }
	else if (p == SRP_PRIM_LINE_STRIP) { out[0] = base + k; out[1] = base + k + 1; }
	else { out[0] = base + k; out[1] = base + (k + 1) % n; }
}

static void warnExcess(SRPPrimitive p, size_t n)
{
	/* src/pipeline/primitive_assembly.c:137-153 */
	if (p == SRP_PRIM_LINES && n % 2 != 0)
		message(SRP_MESSAGE_WARNING, SRP_MESSAGE_SEVERITY_LOW, "warnOnExcessVertexCount",
		        "Odd vertex count when drawing SRP_PRIM_LINES. The last vertex will be ignored\n");
	if (p == SRP_PRIM_TRIANGLES && n % 3 != 0)
		message(SRP_MESSAGE_WARNING, SRP_MESSAGE_SEVERITY_LOW, "warnOnExcessVertexCount",
		        "Vertex count not divisible by 3 when drawing SRP_PRIM_TRIANGLES. The last %i vertex/vertices will be ignored\n",
		        (int) (n % 3));
}

/* Assemble, clip and set up every triangle in submission order, numbering the
 * survivors, then rasterise them in that order
 * (src/pipeline/draw.c:84-125, primitive_assembly.c:37-135). */
static void drawTriangles(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                          const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count)
{
	if (srpContext.raster.cullFace == SRP_FACE_FRONT_AND_BACK) return;
	warnExcess(prim, count);
	size_t nIn = triCount(count, prim);
	if (nIn == 0) return;
	VCache cache;
	cacheInit(&cache, ib, start, count, sp->vs->varyingsSize);
	const SRPPolygonMode mode = srpContext.raster.polygonMode;
	size_t cap = 1024, n = 0;
	Tri* tris = NULL; Line* lines = NULL; Point* pts = NULL;
	size_t id = 0;
	SRPVertexShaderOut clipped[MAX_POLY][3];
	for (size_t k = 0; k < nIn; ++k) {
		size_t s[3];
		triStream(start, k, prim, s);
		SRPVertexShaderOut in[3];
		for (int i = 0; i < 3; ++i) {
			size_t vi = ib ? (size_t) fetchIndex(ib, s[i]) : s[i];
			in[i] = *cacheFetch(&cache, vi, vb, sp);
		}
		size_t nc = clipTri(in, sp, clipped);
		for (size_t c = 0; c < nc; ++c) {
			if (mode == SRP_POLYGON_MODE_FILL) {
				if (!tris || n == cap) { cap = tris ? 2 * cap : cap; tris = (Tri*) realloc(tris, cap * sizeof(Tri)); }
				Tri* t = &tris[n];
				for (int i = 0; i < 3; ++i) t->v[i] = clipped[c][i];
				if (!setupTri(t, fb)) continue;
				t->id = id++;
				++n;
			} else if (mode == SRP_POLYGON_MODE_LINE) {
				for (int j = 0; j < 3; ++j) {
					if (!lines || n == cap) { cap = lines ? 2 * cap : cap; lines = (Line*) realloc(lines, cap * sizeof(Line)); }
					Line* l = &lines[n++];
					l->v[0] = clipped[c][j];
					l->v[1] = clipped[c][(j + 1) % 3];
					setupLn(l, fb);
					l->id = id++;
				}
			} else if (mode == SRP_POLYGON_MODE_POINT) {
				for (int j = 0; j < 3; ++j) {
					if (!pts || n == cap) { cap = pts ? 2 * cap : cap; pts = (Point*) realloc(pts, cap * sizeof(Point)); }
					Point* p = &pts[n++];
					p->v = clipped[c][j];
					perspectiveDivide(&p->v, NULL);
					p->id = id++;
				}
			} else {
				message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "assembleTrianglesGeneric",
				        "Unexpected srpContext.raster.polygonMode (%i)", mode);
			}
		}
	}
	void* interp = xmalloc(sp->vs->varyingsSize + 16);
	for (size_t i = 0; i < n; ++i) {
		if (mode == SRP_POLYGON_MODE_FILL) rasterTri(&tris[i], fb, sp, interp);
		else if (mode == SRP_POLYGON_MODE_LINE) rasterLn(&lines[i], fb, sp, interp);
		else if (mode == SRP_POLYGON_MODE_POINT) rasterPt(&pts[i], fb, sp);
	}
	free(interp); free(tris); free(lines); free(pts);
}

/* src/pipeline/draw.c:127-146, primitive_assembly.c:137-178 */
static void drawLines(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                      const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count)
{
	warnExcess(prim, count);
	size_t nl = lineCount(count, prim);
	if (nl == 0) return;
	Line* lines = (Line*) xmalloc(nl * sizeof(Line));
	VCache cache;
	cacheInit(&cache, ib, start, count, sp->vs->varyingsSize);
	size_t id = 0;
	for (size_t k = 0; k < nl; ++k) {
		Line* l = &lines[id];
		size_t s[2];
		lineStream(start, k, prim, count, s);
		for (int i = 0; i < 2; ++i) {
			size_t vi = ib ? (size_t) fetchIndex(ib, s[i]) : s[i];
			l->v[i] = *cacheFetch(&cache, vi, vb, sp);
		}
		if (clipLineSeg(l->v, sp)) continue;
		setupLn(l, fb);
		l->id = id++;
	}
	void* interp = xmalloc(sp->vs->varyingsSize + 16);
	for (size_t i = 0; i < id; ++i) rasterLn(&lines[i], fb, sp, interp);
	free(interp);
	free(lines);
}

/* src/pipeline/draw.c:148-165, primitive_assembly.c:221-254: no vertex cache */
static void drawPoints(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                       const SRPShaderProgram* sp, size_t start, size_t count)
{
	if (srpContext.raster.pointSize <= 0.) return;
	Point* pts = (Point*) xmalloc(count * sizeof(Point));
	unsigned char* vary = (unsigned char*) scratchAlloc(sp->vs->varyingsSize * count + 1);
	size_t id = 0;
	for (size_t k = 0; k < count; ++k) {
		Point* p = &pts[id];
		size_t vi = ib ? (size_t) fetchIndex(ib, start + k) : start + k;
		runVertexShader(vi, vary + k * sp->vs->varyingsSize, vb, sp, &p->v);
		if (clipPointV(&p->v)) continue;
		perspectiveDivide(&p->v, NULL);
		p->id = id++;
	}
	for (size_t i = 0; i < id; ++i) rasterPt(&pts[i], fb, sp);
	free(pts);
}

/* Range check then dispatch by primitive class (src/pipeline/draw.c:63-82, 167-189). */
static void drawBuffer(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                       const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count)
{
	if (count == 0) return;
	size_t end = start + count - 1;
	size_t size = ib ? ib->nIndices : vb->nVertices;
	if (end >= size) {
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "checkOOB",
		        ib ? "Attempt to OOB access index buffer (read) at indices %zu-%zu (size: %zu)\n"
		           : "Attempt to OOB access vertex buffer (read) at indices %zu-%zu (size: %zu)\n",
		        start, end, size);
		return;
	}
	if (prim == SRP_PRIM_TRIANGLES || prim == SRP_PRIM_TRIANGLE_STRIP || prim == SRP_PRIM_TRIANGLE_FAN)
		drawTriangles(ib, vb, fb, sp, prim, start, count);
	else if (prim == SRP_PRIM_LINES || prim == SRP_PRIM_LINE_STRIP || prim == SRP_PRIM_LINE_LOOP)
		drawLines(ib, vb, fb, sp, prim, start, count);
	else if (prim == SRP_PRIM_POINTS)
		drawPoints(ib, vb, fb, sp, start, count);
	else
		message(SRP_MESSAGE_ERROR, SRP_MESSAGE_SEVERITY_HIGH, "drawBuffer", "Unknown primitive type: %i", prim);
	scratchReset();
}

void srpDrawVertexBuffer(const SRPVertexBuffer* vb, const SRPFramebuffer* fb, const SRPShaderProgram* sp,
                         SRPPrimitive prim, size_t start, size_t count)
{
	drawBuffer(NULL, vb, fb, sp, prim, start, count);
}

void srpDrawIndexBuffer(const SRPIndexBuffer* ib, const SRPVertexBuffer* vb, const SRPFramebuffer* fb,
                        const SRPShaderProgram* sp, SRPPrimitive prim, size_t start, size_t count)
{
	drawBuffer(ib, vb, fb, sp, prim, start, count);
}
