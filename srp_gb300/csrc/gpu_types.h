/* Types shared by the host side of the library and its CUDA kernels. */
#pragma once

#include <stdint.h>
#include <stddef.h>

namespace srpg {

/* Largest user uniform block the GPU path accepts (it travels as a kernel
 * parameter, so shaders read it from the constant bank). */
constexpr int kMaxUniformBytes = 1024;
/* Largest vertex record / varying block handled by the kernels. */
constexpr int kMaxVertexWords = 32;
constexpr int kMaxVaryingWords = 32;
constexpr int kMaxVaryings = 16;
/* Vertices a Sutherland-Hodgman polygon can reach (3 + one per plane). */
constexpr int kMaxPoly = 9;
/* Triangles of the fan of such a polygon. */
constexpr int kClipFan = kMaxPoly - 2;

enum VaryingMode : uint8_t { kPerspective = 0, kAffine = 1, kFlat = 2 };

/* One varying attribute: nItems elements of `type` at byte offset `offset`. */
struct VaryingAttr {
	uint16_t offset;
	uint16_t nItems;
	uint8_t type;        /* SRPType */
	uint8_t mode;        /* VaryingMode */
	uint8_t elemSize;
	uint8_t pad;
};

struct VaryingLayout {
	int nAttr;
	int sizeBytes;
	int nWords;          /* ceil(sizeBytes / 4) */
	int floatOnly;       /* every attribute is 4-byte float/int at a 4-aligned offset */
	VaryingAttr attr[kMaxVaryings];
	uint8_t wordMode[kMaxVaryingWords];   /* floatOnly: per-word VaryingMode */
	uint8_t wordIsFloat[kMaxVaryingWords];
};

struct StencilFace {
	int func, sfail, dfail, pass;
	uint32_t ref, mask, writeMask, pad;
};

/* Pipeline state for one draw (a snapshot of SRPContext plus derived values). */
struct DrawState {
	int W, H;
	int frontFaceCW;
	int cullFace;        /* SRPFace */
	int polygonMode;
	float pointSize;
	int provokingFirst;
	int scissorEnabled;
	uint64_t sx0, sx1, sy0, sy1;   /* [x0, x0 + width) with size_t wrap-around */
	int stencilEnabled;
	int depthTest, depthWrite, depthOp;
	int earlyZ;          /* !mayOverwriteDepth */
	int pad0;
	StencilFace front, back;
	int tile;            /* tile edge in pixels */
	int tilesX, tilesY;
	int pad1;
};

/* Levels of a mip chain kept on the device (textures up to 2^31 texels wide). */
constexpr int kMaxMipLevels = 32;

/* Device texture descriptor (RGBA8 texels, alpha unused: the reference keeps
 * three channels and reads alpha as 1). */
struct TextureDesc {
	const uint32_t* texels;          /* level 0, then the mip levels (TRILINEAR) */
	int width, height, wm1, hm1;
	int wrapX, wrapY;
	int filter;                      /* SRPTextureFilter */
	int nLevels;                     /* levels stored (1 unless TRILINEAR) */
	int lw[kMaxMipLevels], lh[kMaxMipLevels];
	uint32_t loff[kMaxMipLevels];    /* first texel of each level */
};

/* Triangle record read by the tile resolve kernel (64 bytes). */
struct __align__(16) TriRaster {
	float l0[3];         /* barycentrics at the centre of the bbox-min pixel */
	float dx[3], dy[3];  /* per-pixel and per-row increments */
	float c[3];          /* z_ndc * invW per vertex (depth = sum c_i * lambda_i) */
	uint16_t minX, minY, maxX, maxY;   /* bbox, max exclusive */
	uint32_t flags;      /* bit0 front facing, bits1..3 top-left flags */
	uint32_t table;      /* big triangles: offset of their lambda table, else kNoTable */
};

constexpr uint32_t kNoTable = 0xFFFFFFFFu;

/* Triangle data needed only for shading (32 bytes). */
struct __align__(16) TriAttr {
	float invW[3];
	uint32_t vref[3];    /* rows of the post-VS vertex arrays */
	uint32_t id;         /* primitiveID */
	uint32_t pad;
};

/* Line record after setup (48 bytes). */
struct __align__(16) LineRec {
	float x0, y0, xInc, yInc;
	float tInc;
	int32_t steps;
	float c[2];          /* z_ndc * invW */
	float invW[2];
	uint32_t vref[2];
	uint32_t id;
	uint32_t fragBase;   /* first pair slot of its runs */
	uint32_t slots;      /* pair slots of its runs; bit 31: every step lands in the framebuffer */
	uint32_t endPix;     /* pixel one step past the last (x | y << 16, 16 bits each) */
};

/* Line draws bin runs of fragments (k_front.cu): a run's pair value is its
 * slot k | count << kRunCountShift, its fragments' records are at
 * k * kRunFrags + j (a run has at most kRunMaxCount fragments, and slots
 * stay below 2^kRunCountShift). */
constexpr uint32_t kRunFrags = 16;
constexpr uint32_t kRunCountShift = 28;
constexpr uint32_t kRunMaxCount = 15;

/* One line fragment (16 bytes). */
struct __align__(16) LineFrag {
	float depth;
	float t;
	uint32_t line;       /* index into the line records */
	int16_t px, py;      /* logical pixel (px may equal the width) */
};

/* Point record after setup (32 bytes). */
struct __align__(16) PointRec {
	float mnx, mny, mxx, mxy;   /* coverage square, [mn, mx) */
	float z;
	uint32_t vref;
	uint32_t id;
	int16_t x0, y0, x1, y1;     /* raster bounds, inclusive, clamped to the framebuffer */
};

enum PrimKind { kKindTri = 0, kKindLineFrag = 1, kKindPoint = 2 };

/* One draw of a multi-draw pass (srpGpuDrawBatch): the fields in which the
 * draws of one pass differ. State, shaders and varying layout are shared by
 * the pass and stay in DrawParams. */
struct alignas(16) DrawDesc {
	const unsigned char* vertices;   /* device copy of the draw's vertex buffer */
	const void* indices;             /* device copy of its index buffer, or null */
	unsigned long long start, count, nVertices;
	int indexSize, stride;
	int prim;                        /* SRPPrimitive (a triangle topology) */
	int W, H, tilesX, tilesY;
	int pad;
	uint32_t* color;                 /* the draw's framebuffer planes */
	float* depth;
	uint8_t* stencil;
	int32_t* winner;                 /* its part of the pass's winner plane */
	alignas(16) unsigned char uniform[kMaxUniformBytes];
};

/* Counters written by the kernels, read back by the host. */
struct DeviceCounters {
	unsigned long long fragments;
	unsigned long long prims;        /* primitives emitted by setup */
	unsigned long long entries;      /* (tile, primitive) pairs */
	unsigned long long bigJobs;
	unsigned long long clipVerts;    /* clip-generated vertices */
	unsigned long long lineFrags;
	unsigned long long clipOverflow;
	unsigned long long tableWords;   /* floats of lambda tables requested */
	unsigned long long clipTris;     /* triangles clipped by the pre-pass */
	unsigned int errors;             /* bit mask, see kErr* */
	unsigned int lookbackTicket;
	unsigned int nonEmptyTiles;      /* heavy tiles listed by k_tile_classify */
	unsigned int abort;              /* set by k_check: a count exceeded its buffer, skip the rest */
	unsigned int learnedPairs;       /* next tile pair for learned shading's groups to take */
};

enum : unsigned {
	kErrBadIndex = 1u,        /* vertex index outside the vertex buffer */
	kErrCapacity = 2u,        /* a scratch buffer was too small (draw is retried) */
	kErrSpin = 4u,            /* a bounded wait gave up */
	kErrUnsupported = 8u,
};

}  // namespace srpg
