/* Seeded synthetic scenes for parity tests and benchmarks (see scenes.h).
 *
 * Workloads:
 *   sphere      indexed UV sphere, 64 rings x 128 segments (8,385 vertices,
 *               16,128 triangles), random rotation, 60 degree perspective,
 *               near 0.1, far 100, Gouraud colours, CCW back-face culling,
 *               512x512, depth LESS.
 *   soup        random geodesic spheres (5k-50k triangles each, radius
 *               log-uniform 0.05-2, centres in a 20^3 box, about 20% cut by
 *               the near plane) totalling ~2M triangles, a 1024x1024 random
 *               texture, then 100k lines and 100k points; 1920x1080, scissor
 *               = central 80%, stencil INCR on depth pass, depth LESS, mixed
 *               perspective/affine/flat varyings.
 *   plus small feature scenes covering clipping, interpolation modes,
 *   provoking vertex, depth ops, the fill rule, scissor, stencil ops,
 *   polygon modes, all topologies and index types, late depth and fragCoord.
 * `scale` shrinks triangle counts, line/point counts and the framebuffer. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "scenes.h"
#include "srp/mat.h"
#include "srp/shaderlib.h"
#ifdef SCENES_GPU
#include <cuda_runtime_api.h>
#include "srp/gpu.h"
#endif
#ifdef SCENES_REF
#include <unistd.h>
#include "../csrc/imageio.h"
#endif

/* ------------------------------------------------ deterministic numerics */

typedef struct Rng { uint64_t s; } Rng;

static uint64_t rngNext(Rng* r)
{
	/* splitmix64 */
	uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}
static double rngU(Rng* r) { return (double) (rngNext(r) >> 11) * (1.0 / 9007199254740992.0); }
static double rngRange(Rng* r, double a, double b) { return a + (b - a) * rngU(r); }

static const double PI_D = 3.14159265358979323846;

/* sin/cos/exp/log from + - * / only, so that results do not depend on the
 * platform's libm. Accuracy is ~1e-15, determinism is what matters. */
static double dsin(double x)
{
	double k = floor(x / (2 * PI_D) + 0.5);
	double r = x - k * (2 * PI_D);
	if (r > PI_D / 2) r = PI_D - r;
	else if (r < -PI_D / 2) r = -PI_D - r;
	double r2 = r * r, term = r, sum = r;
	for (int n = 1; n < 12; ++n) {
		term = -term * r2 / (double) ((2 * n) * (2 * n + 1));
		sum = sum + term;
	}
	return sum;
}
static double dcos(double x) { return dsin(x + PI_D / 2); }
static double dexp(double x)
{
	double k = floor(x / 0.69314718055994530942 + 0.5);
	double r = x - k * 0.69314718055994530942;
	double term = 1, sum = 1;
	for (int n = 1; n < 20; ++n) { term = term * r / n; sum = sum + term; }
	return ldexp(sum, (int) k);
}
static double dlog(double x)
{
	int e;
	double m = frexp(x, &e);  /* x = m * 2^e, m in [0.5, 1) */
	double z = (m - 1) / (m + 1), z2 = z * z, term = z, sum = z;
	for (int n = 1; n < 30; ++n) { term = term * z2; sum = sum + term / (2 * n + 1); }
	return 2 * sum + e * 0.69314718055994530942;
}
static double logUniform(Rng* r, double a, double b) { return dexp(rngRange(r, dlog(a), dlog(b))); }

/* Rotation about X, then Y, then Z, built with the deterministic sin/cos. */
static mat4 rotation(double ax, double ay, double az)
{
	double sx = dsin(ax), cx = dcos(ax), sy = dsin(ay), cy = dcos(ay), sz = dsin(az), cz = dcos(az);
	mat4 m = mat4ConstructIdentity();
	m.data[0][0] = (float) (cy * cz);
	m.data[0][1] = (float) (sx * sy * cz - cx * sz);
	m.data[0][2] = (float) (cx * sy * cz + sx * sz);
	m.data[1][0] = (float) (cy * sz);
	m.data[1][1] = (float) (sx * sy * sz + cx * cz);
	m.data[1][2] = (float) (cx * sy * sz - sx * cz);
	m.data[2][0] = (float) (-sy);
	m.data[2][1] = (float) (sx * cy);
	m.data[2][2] = (float) (cx * cy);
	return m;
}

/* 60 degree vertical field of view: near-plane half extents near*tan(30). */
static mat4 perspective60(float aspect, float zn, float zf)
{
	const float t = (float) (0.57735026918962576451 * zn);
	return mat4ConstructPerspectiveProjection(-t * aspect, t * aspect, -t, t, zn, zf);
}

static uint64_t fnv(uint64_t h, const void* p, size_t n)
{
	const unsigned char* b = (const unsigned char*) p;
	for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 0x100000001B3ull; }
	return h;
}

/* ------------------------------------------------------------ scene data */

#define MAX_BUF 6
#define MAX_PROG 6

struct Scene {
	char name[32];
	uint64_t seed;
	double scale;
	int W, H;
	float depthInit;
	uint8_t stencilInit;
	int usesStencil;
	void (*render)(Scene*, SRPFramebuffer*);
	/* geometry */
	int nvb, nib;
	SRPVertexBuffer* vb[MAX_BUF];
	void* vdata[MAX_BUF];
	size_t vbytes[MAX_BUF], vstride[MAX_BUF];
	SRPIndexBuffer* ib[MAX_BUF];
	void* idata[MAX_BUF];
	size_t ibytes[MAX_BUF];
	SRPType itype[MAX_BUF];
	/* shading */
	SRPTexture* tex;
	SRPTexture* texExtra[2];   /* more textures of a scene (texfilter) */
	size_t texBytes;
	int nprog;
	SRPStdUniform uni[MAX_PROG];
	SRPVaryingInfo vinfo[MAX_PROG][8];
	SRPVertexShader vs[MAX_PROG];
	SRPFragmentShader fs[MAX_PROG];
	SRPShaderProgram sp[MAX_PROG];
	/* draw list bookkeeping */
	size_t nTris, nLines, nPoints;
	int draws;
	int param[8];
	uint64_t hash;
};

/* Host copies of the scene's buffers. With a GPU they are page-locked, so
 * that the per-frame upload of the end-to-end measurement runs at the host
 * link's speed, as it would for a program that keeps its geometry pinned. */
static void* hostAlloc(size_t nbytes)
{
#ifdef SCENES_GPU
	void* p = NULL;
	if (cudaMallocHost(&p, nbytes ? nbytes : 1) == cudaSuccess) return p;
	fprintf(stderr, "scenes: cudaMallocHost of %zu bytes failed\n", nbytes);
	abort();
#else
	return malloc(nbytes ? nbytes : 1);
#endif
}

static void hostFree(void* p)
{
#ifdef SCENES_GPU
	cudaFreeHost(p);
#else
	free(p);
#endif
}

static int addVB(Scene* s, const void* data, size_t stride, size_t nbytes)
{
	int k = s->nvb++;
	s->vdata[k] = hostAlloc(nbytes);
	memcpy(s->vdata[k], data, nbytes);
	s->vbytes[k] = nbytes;
	s->vstride[k] = stride;
	s->vb[k] = srpNewVertexBuffer();
	srpVertexBufferCopyData(s->vb[k], stride, nbytes, s->vdata[k]);
	s->hash = fnv(s->hash, data, nbytes);
	return k;
}

static int addIB(Scene* s, SRPType type, const void* data, size_t nbytes)
{
	int k = s->nib++;
	s->idata[k] = hostAlloc(nbytes);
	memcpy(s->idata[k], data, nbytes);
	s->ibytes[k] = nbytes;
	s->itype[k] = type;
	s->ib[k] = srpNewIndexBuffer();
	srpIndexBufferCopyData(s->ib[k], type, nbytes, s->idata[k]);
	s->hash = fnv(s->hash, data, nbytes);
	return k;
}

static SRPTexture* makeTexture(Scene* s, const uint8_t* rgb, int w, int h,
                               SRPTextureWrappingMode wx, SRPTextureWrappingMode wy)
{
	s->hash = fnv(s->hash, rgb, (size_t) w * h * 3);
	s->texBytes = (size_t) w * h * 3;
#ifdef SCENES_REF
	/* The reference loads textures from files only. */
	char path[128];
	snprintf(path, sizeof path, "/tmp/srp_scene_tex_%d.ppm", (int) getpid());
	srpImageWritePPM(path, rgb, w, h);
	SRPTexture* t = srpNewTexture(path, wx, wy);
	remove(path);
	return t;
#else
	return srpNewTextureFromMemory(rgb, w, h, 3, wx, wy);
#endif
}

/* Program k: vertex shader, fragment shader and varying layout. */
static SRPShaderProgram* program(Scene* s, int k,
                                 void (*vs)(SRPVertexShaderIn*, SRPVertexShaderOut*),
                                 void (*fs)(SRPFragmentShaderIn*, SRPFragmentShaderOut*),
                                 int mayOverwriteDepth, int nvary, const SRPVaryingInfo* info)
{
	if (k >= s->nprog) s->nprog = k + 1;
	size_t size = 0;
	for (int i = 0; i < nvary; ++i) {
		s->vinfo[k][i] = info[i];
		size_t es = (info[i].type == SRP_DOUBLE || info[i].type == SRP_INT64 || info[i].type == SRP_UINT64) ? 8
		          : (info[i].type == SRP_INT16 || info[i].type == SRP_UINT16) ? 2
		          : (info[i].type == SRP_INT8 || info[i].type == SRP_UINT8) ? 1 : 4;
		size += es * info[i].nItems;
	}
	s->vs[k].shader = vs;
	s->vs[k].nVaryings = (size_t) nvary;
	s->vs[k].varyingsInfo = nvary ? s->vinfo[k] : NULL;
	s->vs[k].varyingsSize = size;
	s->fs[k].shader = fs;
	s->fs[k].mayOverwriteDepth = mayOverwriteDepth != 0;
	s->sp[k].uniform = (SRPUniform*) &s->uni[k];
	s->sp[k].vs = &s->vs[k];
	s->sp[k].fs = &s->fs[k];
	return &s->sp[k];
}

static void hashUniforms(Scene* s)
{
	for (int k = 0; k < s->nprog; ++k)
		s->hash = fnv(s->hash, &s->uni[k], offsetof(SRPStdUniform, texture));
}

static SRPVaryingInfo vi(size_t n, SRPType t, SRPInterpolationMode m)
{
	SRPVaryingInfo v;
	v.nItems = n; v.type = t; v.interpolationMode = m;
	return v;
}

#ifdef SCENES_GPU
/* With the switch on, every draw of a scene goes through
 * srpGpuDrawFixedScratch instead; rejected draws are counted. */
static int gFixedScratch, gFixedRejected;
void sceneUseFixedScratch(int on) { gFixedScratch = on; gFixedRejected = 0; }
int sceneFixedScratchRejected(void) { return gFixedRejected; }
#endif

static void drawI(Scene* s, int ib, int vb, SRPFramebuffer* fb, int prog, SRPPrimitive p, size_t start, size_t count)
{
#ifdef SCENES_GPU
	if (gFixedScratch) {
		gFixedRejected += srpGpuDrawFixedScratch(s->ib[ib], s->vb[vb], fb, &s->sp[prog], p, start, count) != 0;
		return;
	}
#endif
	srpDrawIndexBuffer(s->ib[ib], s->vb[vb], fb, &s->sp[prog], p, start, count);
}

static void drawV(Scene* s, int vb, SRPFramebuffer* fb, int prog, SRPPrimitive p, size_t start, size_t count)
{
#ifdef SCENES_GPU
	if (gFixedScratch) {
		gFixedRejected += srpGpuDrawFixedScratch(NULL, s->vb[vb], fb, &s->sp[prog], p, start, count) != 0;
		return;
	}
#endif
	srpDrawVertexBuffer(s->vb[vb], fb, &s->sp[prog], p, start, count);
}

static void baseUniform(SRPStdUniform* u)
{
	memset(u, 0, sizeof *u);
	u->model = mat4ConstructIdentity();
	u->view = mat4ConstructIdentity();
	u->projection = mat4ConstructIdentity();
	for (int k = 0; k < 4; ++k) { u->color[k] = 1.f; u->ambient[k] = 0.15f; }
	u->shininess = 64.f;
	u->marbleFrequency = 4.f;
	u->marbleGain = 0.5f;
	u->marbleOctaves = 8;
	u->depthScale = 0.5f;
	u->depthBias = 0.f;
}

/* ---------------------------------------------------------- mesh builders */

typedef struct Mesh { float* v; size_t nv, stride; uint32_t* idx; size_t ni; } Mesh;

/* UV sphere: (rings + 1) x (segs + 1) vertices (seam duplicated for uv),
 * pole bands emit one triangle per segment. Layout: pos3 normal3 uv2 rgb3. */
static Mesh uvSphere(int rings, int segs, Rng* rng, float radius)
{
	Mesh m;
	m.stride = 11;
	m.nv = (size_t) (rings + 1) * (segs + 1);
	m.v = (float*) malloc(m.nv * m.stride * sizeof(float));
	for (int i = 0; i <= rings; ++i) {
		double th = PI_D * i / rings;
		for (int j = 0; j <= segs; ++j) {
			double ph = 2 * PI_D * j / segs;
			float* p = m.v + ((size_t) i * (segs + 1) + j) * m.stride;
			double nx = dsin(th) * dcos(ph), ny = dcos(th), nz = dsin(th) * dsin(ph);
			p[0] = (float) (radius * nx); p[1] = (float) (radius * ny); p[2] = (float) (radius * nz);
			p[3] = (float) nx; p[4] = (float) ny; p[5] = (float) nz;
			p[6] = (float) j / segs; p[7] = 1.f - (float) i / rings;
			p[8] = (float) rngU(rng); p[9] = (float) rngU(rng); p[10] = (float) rngU(rng);
		}
	}
	m.idx = (uint32_t*) malloc((size_t) rings * segs * 6 * sizeof(uint32_t));
	m.ni = 0;
	for (int i = 0; i < rings; ++i)
		for (int j = 0; j < segs; ++j) {
			uint32_t a = (uint32_t) (i * (segs + 1) + j), b = a + 1;
			uint32_t c = (uint32_t) ((i + 1) * (segs + 1) + j), d = c + 1;
			/* counter-clockwise seen from outside once projected */
			if (i != 0) { m.idx[m.ni++] = a; m.idx[m.ni++] = b; m.idx[m.ni++] = c; }
			if (i != rings - 1) { m.idx[m.ni++] = b; m.idx[m.ni++] = d; m.idx[m.ni++] = c; }
		}
	return m;
}

static void freeMesh(Mesh* m) { free(m->v); free(m->idx); }

/* Geodesic sphere: each icosahedron face split into f*f triangles, points
 * pushed to the sphere. 20*f*f triangles, (f+1)(f+2)/2 vertices per face. */
static const int ICO_F[20][3] = {
	{0,11,5},{0,5,1},{0,1,7},{0,7,10},{0,10,11},{1,5,9},{5,11,4},{11,10,2},{10,7,6},{7,1,8},
	{3,9,4},{3,4,2},{3,2,6},{3,6,8},{3,8,9},{4,9,5},{2,4,11},{6,2,10},{8,6,7},{9,8,1}};

static void icoVertex(int i, double* p)
{
	const double g = (1.0 + sqrt(5.0)) / 2.0;
	static const signed char T[12][3] = {
		{-1,1,0},{1,1,0},{-1,-1,0},{1,-1,0},{0,-1,1},{0,1,1},{0,-1,-1},{0,1,-1},{1,0,-1},{1,0,1},{-1,0,-1},{-1,0,1}};
	/* (a, b*g, 0) cyclic pattern */
	double a = T[i][0], b = T[i][1], c = T[i][2];
	if (i < 4) { p[0] = a; p[1] = b * g; p[2] = 0; }
	else if (i < 8) { p[0] = 0; p[1] = b; p[2] = c * g; }
	else { p[0] = a * g; p[1] = 0; p[2] = c; }
}

/* Appends a geodesic sphere to (verts, idx). Layout: pos3 normal3 uv2 rgb3 id1. */
static void appendGeodesic(float** verts, size_t* nv, size_t* capv, uint32_t** idx, size_t* ni, size_t* capi,
                           int f, const double* centre, double radius, uint32_t meshId, Rng* rng)
{
	const size_t stride = 12;
	size_t addV = (size_t) 20 * (f + 1) * (f + 2) / 2, addI = (size_t) 20 * f * f * 3;
	while (*nv + addV > *capv) { *capv = *capv ? *capv * 2 : 1 << 16; *verts = (float*) realloc(*verts, *capv * stride * sizeof(float)); }
	while (*ni + addI > *capi) { *capi = *capi ? *capi * 2 : 1 << 16; *idx = (uint32_t*) realloc(*idx, *capi * sizeof(uint32_t)); }
	/* one draw per statement: C leaves the order of evaluation of function
	 * arguments and initialiser-list elements unspecified */
	float tint[3];
	for (int k = 0; k < 3; ++k) tint[k] = (float) rngRange(rng, 0.4, 1);
	for (int fc = 0; fc < 20; ++fc) {
		double A[3], B[3], C[3];
		icoVertex(ICO_F[fc][0], A); icoVertex(ICO_F[fc][1], B); icoVertex(ICO_F[fc][2], C);
		size_t base = *nv;
		for (int i = 0; i <= f; ++i)
			for (int j = 0; j <= f - i; ++j) {
				double u = (double) i / f, v = (double) j / f, w = 1 - u - v;
				double p[3];
				for (int k = 0; k < 3; ++k) p[k] = A[k] * w + B[k] * u + C[k] * v;
				double len = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
				float* o = *verts + (*nv) * stride;
				for (int k = 0; k < 3; ++k) {
					o[3 + k] = (float) (p[k] / len);
					o[k] = (float) (centre[k] + radius * p[k] / len);
				}
				o[6] = (float) u; o[7] = (float) v;
				o[8] = tint[0] * (float) (0.7 + 0.3 * w);
				o[9] = tint[1] * (float) (0.7 + 0.3 * u);
				o[10] = tint[2] * (float) (0.7 + 0.3 * v);
				memcpy(&o[11], &meshId, 4);
				++*nv;
			}
		/* index of (i, j) inside this face's triangular grid */
		#define GI(i, j) ((uint32_t) (base + (size_t) (i) * (f + 1) - (size_t) (i) * ((i) - 1) / 2 + (j)))
		for (int i = 0; i < f; ++i)
			for (int j = 0; j < f - i; ++j) {
				uint32_t a = GI(i, j), b = GI(i + 1, j), c = GI(i, j + 1);
				(*idx)[(*ni)++] = a; (*idx)[(*ni)++] = c; (*idx)[(*ni)++] = b;
				if (j < f - i - 1) {
					uint32_t d = GI(i + 1, j + 1);
					(*idx)[(*ni)++] = b; (*idx)[(*ni)++] = c; (*idx)[(*ni)++] = d;
				}
			}
		#undef GI
	}
}

/* ------------------------------------------------------------------ scenes */

static void renderSphere(Scene* s, SRPFramebuffer* fb)
{
	srpRasterFrontFace(SRP_WINDING_CCW);
	srpRasterCullFace(SRP_FACE_BACK);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
}

static void buildSphere(Scene* s, Rng* rng)
{
	int rings = 64, segs = 128;
	s->W = s->H = 512;
	if (s->scale < 1.0) {
		int side = (int) (512 * s->scale);
		s->W = s->H = side < 32 ? 32 : side;
		rings = (int) (64 * s->scale); segs = (int) (128 * s->scale);
		if (rings < 4) rings = 4;
		if (segs < 8) segs = 8;
	}
	Mesh m = uvSphere(rings, segs, rng, 1.0f);
	addVB(s, m.v, m.stride * 4, m.nv * m.stride * 4);
	addIB(s, SRP_UINT32, m.idx, m.ni * 4);
	s->nTris = m.ni / 3;
	freeMesh(&m);
	SRPStdUniform* u = &s->uni[0];
	baseUniform(u);
	double ang[3];
	for (int k = 0; k < 3; ++k) ang[k] = rngRange(rng, 0, 2 * PI_D);
	u->model = rotation(ang[0], ang[1], ang[2]);
	u->view = mat4ConstructTranslate(0, 0, 3);
	u->projection = perspective60((float) s->W / (float) s->H, 0.1f, 100.f);
	u->passOffset = 8; u->passCount = 3;  /* Gouraud rgb */
	SRPVaryingInfo v[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v);
	s->depthInit = 1.0f;
	s->render = renderSphere;
	s->draws = 1;
}

static void renderSoup(Scene* s, SRPFramebuffer* fb)
{
	srpRasterFrontFace(SRP_WINDING_CCW);
	srpRasterCullFace(SRP_FACE_BACK);
	srpRasterPointSize(2.f);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	srpScissorTest(true);
	srpScissorOptions((size_t) (s->W / 10), (size_t) (s->H / 10), (size_t) (s->W * 8 / 10), (size_t) (s->H * 8 / 10));
	srpStencilTest(true);
	srpStencilFunc(SRP_COMPARE_ALWAYS, 0, 0xFF);
	srpStencilOp(SRP_STENCIL_KEEP, SRP_STENCIL_KEEP, SRP_STENCIL_INCR);
	srpStencilWriteMask(0xFF);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
	if (s->nLines) drawV(s, 1, fb, 1, SRP_PRIM_LINES, 0, 2 * s->nLines);
	if (s->nPoints) drawV(s, 2, fb, 1, SRP_PRIM_POINTS, 0, s->nPoints);
}

static void buildSoup(Scene* s, Rng* rng)
{
	s->W = 1920; s->H = 1080;
	if (s->scale < 1.0) {
		double lin = sqrt(s->scale);
		s->W = (int) (1920 * lin) & ~7; s->H = (int) (1080 * lin) & ~7;
		if (s->W < 64) s->W = 64;
		if (s->H < 48) s->H = 48;
	}
	const size_t target = (size_t) (2000000 * s->scale);
	float* verts = NULL; uint32_t* idx = NULL;
	size_t nv = 0, ni = 0, capv = 0, capi = 0;
	uint32_t meshId = 0;
	while (ni / 3 < target) {
		double tris = logUniform(rng, 5000, 50000);
		int f = (int) floor(sqrt(tris / 20) + 0.5);
		if (s->scale < 0.05 && f > 12) f = 4 + (int) (rngU(rng) * 8);
		double r = logUniform(rng, 0.05, 2.0);
		double c[3];
		if (rngU(rng) < 0.2) {
			/* cut by the near plane (view z = 0.1) with the eye outside the sphere */
			double zc = 0.1 + r * rngRange(rng, -0.5, 0.5);
			double rho = sqrt(fmax(0.0, 1.2 * r * r - zc * zc)) + r * rngRange(rng, 0.0, 0.4);
			double ang = rngRange(rng, 0, 2 * PI_D);
			c[0] = rho * dcos(ang); c[1] = rho * dsin(ang); c[2] = zc;
		} else {
			c[0] = rngRange(rng, -10, 10); c[1] = rngRange(rng, -10, 10); c[2] = rngRange(rng, 0.5, 20.5);
		}
		appendGeodesic(&verts, &nv, &capv, &idx, &ni, &capi, f, c, r, meshId++, rng);
	}
	addVB(s, verts, 48, nv * 48);
	addIB(s, SRP_UINT32, idx, ni * 4);
	s->nTris = ni / 3;
	free(verts); free(idx);

	/* 1024^2 random texture */
	int tw = s->scale < 0.05 ? 64 : 1024;
	uint8_t* tex = (uint8_t*) malloc((size_t) tw * tw * 3);
	for (size_t i = 0; i < (size_t) tw * tw * 3; ++i) tex[i] = (uint8_t) (rngNext(rng) >> 56);
	s->tex = makeTexture(s, tex, tw, tw, TW_REPEAT, TW_REPEAT);
	free(tex);

	/* lines and points: pos3 rgb3 */
	s->nLines = (size_t) (100000 * s->scale);
	s->nPoints = (size_t) (100000 * s->scale);
	float* lv = (float*) malloc((2 * s->nLines + 1) * 6 * sizeof(float));
	for (size_t i = 0; i < s->nLines; ++i) {
		float* a = lv + 12 * i;
		double p[3], d[3];
		p[0] = rngRange(rng, -10, 10); p[1] = rngRange(rng, -10, 10); p[2] = rngRange(rng, 0.2, 20.5);
		for (int k = 0; k < 3; ++k) d[k] = rngRange(rng, -1, 1);
		double len = rngRange(rng, 0.05, 1.0);
		for (int k = 0; k < 3; ++k) { a[k] = (float) p[k]; a[6 + k] = (float) (p[k] + len * d[k]); }
		for (int k = 0; k < 3; ++k) { a[3 + k] = (float) rngU(rng); a[9 + k] = (float) rngU(rng); }
	}
	addVB(s, lv, 24, 2 * s->nLines * 24);
	free(lv);
	float* pv = (float*) malloc((s->nPoints + 1) * 6 * sizeof(float));
	for (size_t i = 0; i < s->nPoints; ++i) {
		float* a = pv + 6 * i;
		a[0] = (float) rngRange(rng, -10, 10); a[1] = (float) rngRange(rng, -10, 10); a[2] = (float) rngRange(rng, 0.2, 20.5);
		a[3] = (float) rngU(rng); a[4] = (float) rngU(rng); a[5] = (float) rngU(rng);
	}
	addVB(s, pv, 24, s->nPoints * 24);
	free(pv);

	mat4 proj = perspective60((float) s->W / (float) s->H, 0.1f, 100.f);
	SRPStdUniform* u = &s->uni[0];
	baseUniform(u);
	u->projection = proj;
	u->passOffset = 6; u->passCount = 6;  /* uv, rgb, mesh id */
	u->texture = s->tex;
	SRPVaryingInfo v0[3] = { vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_AFFINE),
	                         vi(1, SRP_UINT32, SRP_INTERPOLATION_MODE_FLAT) };
	program(s, 0, srpVsTransform, srpFsTextureModulate, 0, 3, v0);
	SRPStdUniform* u1 = &s->uni[1];
	baseUniform(u1);
	u1->projection = proj;
	u1->passOffset = 3; u1->passCount = 3;
	SRPVaryingInfo v1[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 1, srpVsTransform, srpFsVaryingColor, 0, 1, v1);
	s->depthInit = 1.0f;
	s->usesStencil = 1;
	s->render = renderSoup;
	s->draws = 1 + (s->nLines > 0) + (s->nPoints > 0);
}

/* Feature scenes share a 256x192 framebuffer (scaled) and a small helper
 * vertex layout pos3 rgb3 uv2 (8 words). */
static void featureSize(Scene* s) { s->W = 256; s->H = 192; }

static void randomTris(Rng* rng, float* v, size_t n, double spread, double zmin, double zmax, int words)
{
	for (size_t t = 0; t < n; ++t) {
		double c[3];
		c[0] = rngRange(rng, -spread, spread); c[1] = rngRange(rng, -spread, spread); c[2] = rngRange(rng, zmin, zmax);
		double size = rngRange(rng, 0.05, 1.5);
		for (int k = 0; k < 3; ++k) {
			float* p = v + (t * 3 + k) * words;
			p[0] = (float) (c[0] + size * rngRange(rng, -1, 1));
			p[1] = (float) (c[1] + size * rngRange(rng, -1, 1));
			p[2] = (float) (c[2] + size * rngRange(rng, -1, 1));
			p[3] = (float) rngU(rng); p[4] = (float) rngU(rng); p[5] = (float) rngU(rng);
			p[6] = (float) rngRange(rng, -0.5, 1.5); p[7] = (float) rngRange(rng, -0.5, 1.5);
		}
	}
}

static void renderClipTris(Scene* s, SRPFramebuffer* fb)
{
	srpRasterCullFace(SRP_FACE_NONE);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, 3 * s->nTris);
	srpRasterCullFace(SRP_FACE_FRONT);
	srpDepthCompareOp(SRP_COMPARE_LEQUAL);
	drawV(s, 0, fb, 1, SRP_PRIM_TRIANGLES, 0, 3 * s->nTris);
}

/* Large triangles around the eye crossing every frustum plane, including
 * near and far; fragment colour encodes the post-clip primitive number. */
static void buildClipTris(Scene* s, Rng* rng)
{
	featureSize(s);
	s->nTris = (size_t) (400 * (s->scale < 1 ? s->scale : 1)) + 8;
	float* v = (float*) malloc(s->nTris * 3 * 8 * sizeof(float));
	randomTris(rng, v, s->nTris, 3.0, -1.0, 12.0, 8);
	addVB(s, v, 32, s->nTris * 3 * 32);
	free(v);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->model = rotation(0.1 * k, 0.2, 0.05);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 10.f);
		u->passOffset = 3; u->passCount = 5;
	}
	SRPVaryingInfo v0[2] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE), vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_AFFINE) };
	program(s, 0, srpVsTransform, srpFsPrimitiveId, 0, 2, v0);
	program(s, 1, srpVsTransform, srpFsVaryingColor, 0, 2, v0);
	s->depthInit = 1.0f;
	s->render = renderClipTris;
	s->draws = 2;
}

static void renderClipLines(Scene* s, SRPFramebuffer* fb)
{
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_LINES, 0, 2 * s->nLines);
	srpProvokingVertexMode(SRP_PROVOKING_VERTEX_FIRST);
	drawI(s, 0, 0, fb, 1, SRP_PRIM_LINE_STRIP, 0, s->nLines);
	srpDepthTest(false);
	drawV(s, 0, fb, 1, SRP_PRIM_LINE_LOOP, 0, 64 < 2 * s->nLines ? 64 : 2 * s->nLines);
}

/* Long lines crossing the frustum (Liang-Barsky path), indexed with u16. */
static void buildClipLines(Scene* s, Rng* rng)
{
	featureSize(s);
	s->nLines = (size_t) (300 * (s->scale < 1 ? s->scale : 1)) + 8;
	size_t nv = 2 * s->nLines;
	float* v = (float*) malloc(nv * 8 * sizeof(float));
	for (size_t i = 0; i < nv; ++i) {
		float* p = v + 8 * i;
		p[0] = (float) rngRange(rng, -6, 6); p[1] = (float) rngRange(rng, -5, 5); p[2] = (float) rngRange(rng, -2, 14);
		p[3] = (float) rngU(rng); p[4] = (float) rngU(rng); p[5] = (float) rngU(rng);
		p[6] = (float) rngU(rng); p[7] = (float) rngU(rng);
	}
	addVB(s, v, 32, nv * 32);
	free(v);
	uint16_t* idx = (uint16_t*) malloc(nv * sizeof(uint16_t));
	for (size_t i = 0; i < nv; ++i) idx[i] = (uint16_t) ((i * 7919) % nv);
	addIB(s, SRP_UINT16, idx, nv * 2);
	free(idx);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 12.f);
		u->passOffset = 3; u->passCount = 3;
	}
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	SRPVaryingInfo v1[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_FLAT) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsVaryingColor, 0, 1, v1);
	s->depthInit = 1.0f;
	s->render = renderClipLines;
	s->draws = 3;
}

static void renderPoints(Scene* s, SRPFramebuffer* fb)
{
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	srpRasterPointSize(3.f);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_POINTS, 0, s->nPoints);
	srpRasterPointSize(1.f);
	drawV(s, 0, fb, 1, SRP_PRIM_POINTS, 0, s->nPoints);
	srpRasterPointSize(5.5f);
	drawV(s, 0, fb, 0, SRP_PRIM_POINTS, 0, s->nPoints / 4);
}

/* Points inside and outside the frustum (whole-point reject), three sizes,
 * indexed with u64. */
static void buildPoints(Scene* s, Rng* rng)
{
	featureSize(s);
	s->nPoints = (size_t) (2000 * (s->scale < 1 ? s->scale : 1)) + 16;
	float* v = (float*) malloc(s->nPoints * 8 * sizeof(float));
	for (size_t i = 0; i < s->nPoints; ++i) {
		float* p = v + 8 * i;
		p[0] = (float) rngRange(rng, -7, 7); p[1] = (float) rngRange(rng, -6, 6); p[2] = (float) rngRange(rng, -1, 14);
		p[3] = (float) rngU(rng); p[4] = (float) rngU(rng); p[5] = (float) rngU(rng);
		p[6] = 0; p[7] = 0;
	}
	addVB(s, v, 32, s->nPoints * 32);
	free(v);
	uint64_t* idx = (uint64_t*) malloc(s->nPoints * sizeof(uint64_t));
	for (size_t i = 0; i < s->nPoints; ++i) idx[i] = (uint64_t) (s->nPoints - 1 - i);
	addIB(s, SRP_UINT64, idx, s->nPoints * 8);
	free(idx);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 12.f);
		u->passOffset = 3; u->passCount = 3;
	}
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsPrimitiveId, 0, 1, v0);
	s->depthInit = 1.0f;
	s->render = renderPoints;
	s->draws = 3;
}

static void renderInterp(Scene* s, SRPFramebuffer* fb)
{
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	srpRasterCullFace(SRP_FACE_NONE);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, 6);   /* perspective uv */
	drawI(s, 0, 0, fb, 1, SRP_PRIM_TRIANGLES, 6, 6);   /* affine uv */
	srpProvokingVertexMode(SRP_PROVOKING_VERTEX_FIRST);
	drawI(s, 0, 0, fb, 2, SRP_PRIM_TRIANGLES, 12, 6);  /* flat int, first vertex */
	srpProvokingVertexMode(SRP_PROVOKING_VERTEX_LAST);
	drawI(s, 0, 0, fb, 2, SRP_PRIM_TRIANGLES, 18, 6);  /* flat int, last vertex */
	drawI(s, 0, 0, fb, 3, SRP_PRIM_TRIANGLES, 24, 6);  /* fragCoord */
}

#ifndef SCENES_REF
/* Texture filtering (an addition: the reference samples the nearest texel
 * only): three floors receding from z = 1.2 to 40, textured 2 x 10 times
 * over with one 96 x 64 texture (repeat in u, clamp in v), sampled nearest,
 * bilinearly, and trilinearly at a level of detail growing with w
 * (srpFsTextureLod). */
static void renderTexFilter(Scene* s, SRPFramebuffer* fb)
{
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	srpRasterCullFace(SRP_FACE_NONE);
	const size_t n = s->ibytes[0] / 4 / 3;
	for (int k = 0; k < 3; ++k) drawI(s, 0, 0, fb, k, SRP_PRIM_TRIANGLES, (size_t) k * n, n);
}

static void buildTexFilter(Scene* s, Rng* rng)
{
	featureSize(s);
	enum { G = 12 };   /* quads per floor side */
	float* v = (float*) malloc(sizeof(float) * 5 * 3 * (G + 1) * (G + 1));
	uint32_t* idx = (uint32_t*) malloc(sizeof(uint32_t) * 3 * 3 * 6 * G * G);
	size_t nv = 0, ni = 0;
	for (int f = 0; f < 3; ++f) {
		const uint32_t base = (uint32_t) nv;
		const double x0 = -1.9 + 1.3 * f + 0.05 * rngRange(rng, -1, 1);
		for (int j = 0; j <= G; ++j)
			for (int i = 0; i <= G; ++i) {
				float* p = v + 5 * nv++;
				const double a = (double) i / G, b = (double) j / G;
				const double z = 1.2 * pow(40.0 / 1.2, b);
				p[0] = (float) (x0 + 1.2 * a); p[1] = -0.8f; p[2] = (float) z;
				p[3] = (float) (2.0 * a); p[4] = (float) (10.0 * b + 0.02 * f);
			}
		for (int j = 0; j < G; ++j)
			for (int i = 0; i < G; ++i) {
				const uint32_t q = base + (uint32_t) (j * (G + 1) + i);
				const uint32_t t[6] = { q, q + 1, q + G + 2, q, q + G + 2, q + G + 1 };
				memcpy(idx + ni, t, sizeof t);
				ni += 6;
			}
	}
	addVB(s, v, 20, nv * 20);
	addIB(s, SRP_UINT32, idx, ni * 4);
	free(v); free(idx);
	const int tw = 96, th = 64;
	uint8_t* tex = (uint8_t*) malloc((size_t) tw * th * 3);
	for (int y = 0; y < th; ++y)
		for (int x = 0; x < tw; ++x)
			for (int c = 0; c < 3; ++c) {
				const int check = ((x / 8) ^ (y / 8)) & 1;
				tex[3 * (y * tw + x) + c] = (uint8_t) ((check ? 200 : 40) + (int) (rngNext(rng) >> 59) * (c + 1));
			}
	s->tex = makeTexture(s, tex, tw, th, TW_REPEAT, TW_CLAMP_TO_EDGE);
	s->texExtra[0] = makeTexture(s, tex, tw, th, TW_REPEAT, TW_CLAMP_TO_EDGE);
	s->texExtra[1] = makeTexture(s, tex, tw, th, TW_REPEAT, TW_CLAMP_TO_EDGE);
	free(tex);
	srpTextureSetFilter(s->texExtra[0], SRP_TEXTURE_FILTER_BILINEAR);
	srpTextureSetFilter(s->texExtra[1], SRP_TEXTURE_FILTER_TRILINEAR);
	SRPVaryingInfo vp[1] = { vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	for (int k = 0; k < 3; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 60.f);
		u->passOffset = 3; u->passCount = 2;
		u->texelScale = 0.45f + 0.05f * (float) rngU(rng);
		u->texture = k == 0 ? s->tex : s->texExtra[k - 1];
	}
	program(s, 0, srpVsTransform, srpFsTexture, 0, 1, vp);
	program(s, 1, srpVsTransform, srpFsTexture, 0, 1, vp);
	program(s, 2, srpVsTransform, srpFsTextureLod, 0, 1, vp);
	s->depthInit = 1.0f;
	s->render = renderTexFilter;
	s->draws = 3;
}
#endif

/* Four tilted quads (perspective uv, affine uv, flat int with first and last
 * provoking vertex, fragCoord); texture 64x48 with repeat/clamp wrapping. */
static void buildInterp(Scene* s, Rng* rng)
{
	featureSize(s);
	float v[20 * 9];
	for (int q = 0; q < 5; ++q) {
		double cx = -1.6 + 0.8 * q, cy = (q & 1) ? 0.4 : -0.4;
		for (int k = 0; k < 4; ++k) {
			float* p = v + (q * 4 + k) * 9;
			double x = (k == 1 || k == 2) ? 0.5 : -0.5, y = (k >= 2) ? 0.6 : -0.6;
			p[0] = (float) (cx + x * 0.8); p[1] = (float) (cy + y); p[2] = (float) (3.0 + 2.2 * y + 0.3 * x);
			p[3] = (float) ((k == 1 || k == 2) ? 2.3 : -0.7); p[4] = (float) (k >= 2 ? 1.8 : -0.4);
			p[5] = (float) rngU(rng); p[6] = (float) rngU(rng); p[7] = (float) rngU(rng);
			int32_t id = (int32_t) (rngNext(rng) % 1000) - 500;
			memcpy(&p[8], &id, 4);
		}
	}
	addVB(s, v, 36, sizeof v);
	uint8_t idx[30];
	for (int q = 0; q < 5; ++q) {
		uint8_t b = (uint8_t) (4 * q);
		uint8_t t[6] = { b, (uint8_t) (b + 1), (uint8_t) (b + 2), b, (uint8_t) (b + 2), (uint8_t) (b + 3) };
		memcpy(idx + 6 * q, t, 6);
	}
	addIB(s, SRP_UINT8, idx, sizeof idx);
	uint8_t* tex = (uint8_t*) malloc(64 * 48 * 3);
	for (int i = 0; i < 64 * 48 * 3; ++i) tex[i] = (uint8_t) (rngNext(rng) >> 56);
	s->tex = makeTexture(s, tex, 64, 48, TW_REPEAT, TW_CLAMP_TO_EDGE);
	free(tex);
	for (int k = 0; k < 4; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 20.f);
		u->passOffset = 3; u->passCount = 6;
		u->texture = s->tex;
	}
	s->uni[2].varyingOffset = 5;
	SRPVaryingInfo vp[3] = { vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(1, SRP_INT32, SRP_INTERPOLATION_MODE_FLAT) };
	SRPVaryingInfo va[3] = { vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_AFFINE),
	                         vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_AFFINE),
	                         vi(1, SRP_INT32, SRP_INTERPOLATION_MODE_FLAT) };
	program(s, 0, srpVsTransform, srpFsTexture, 0, 3, vp);
	program(s, 1, srpVsTransform, srpFsTexture, 0, 3, va);
	program(s, 2, srpVsTransform, srpFsFlatInt, 0, 3, vp);
	program(s, 3, srpVsTransform, srpFsFragCoord, 0, 3, vp);
	s->depthInit = 1.0f;
	s->render = renderInterp;
	s->draws = 5;
}

static void renderDepthOps(Scene* s, SRPFramebuffer* fb)
{
	srpDepthTest(true);
	srpRasterCullFace(SRP_FACE_NONE);
	for (int op = 0; op < 8; ++op) {
		srpDepthCompareOp((SRPCompareOp) op);
		srpDepthWrite(op != 5);
		drawV(s, 0, fb, op & 1, SRP_PRIM_TRIANGLES, (size_t) op * 3 * s->param[0], 3 * (size_t) s->param[0]);
	}
	srpDepthTest(false);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, 3 * (size_t) s->param[0]);
}

/* Overlapping triangles drawn once per compare op (NEVER..NOTEQUAL), with the
 * depth write switched off for one op, then once with the test disabled. */
static void buildDepthOps(Scene* s, Rng* rng)
{
	featureSize(s);
	int per = 24;
	s->param[0] = per;
	s->nTris = 8 * (size_t) per;
	float* v = (float*) malloc(s->nTris * 3 * 8 * sizeof(float));
	randomTris(rng, v, s->nTris, 1.2, 2.0, 6.0, 8);
	addVB(s, v, 32, s->nTris * 3 * 32);
	free(v);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 20.f);
		u->passOffset = 3; u->passCount = 3;
	}
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsPrimitiveId, 0, 1, v0);
	s->depthInit = 0.2f;
	s->render = renderDepthOps;
	s->draws = 9;
}

static void renderRules(Scene* s, SRPFramebuffer* fb)
{
	srpRasterCullFace(SRP_FACE_NONE);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, 3 * s->nTris);
	srpRasterFrontFace(SRP_WINDING_CW);
	srpRasterCullFace(SRP_FACE_BACK);
	drawV(s, 0, fb, 1, SRP_PRIM_TRIANGLES, 0, 3 * s->nTris);
}

/* Fill-rule torture: a fan of triangles whose shared vertices and edges sit
 * exactly on pixel centres and pixel edges, axis-aligned edges, slivers,
 * sub-pixel and degenerate triangles, orthographic projection. */
static void buildRules(Scene* s, Rng* rng)
{
	featureSize(s);
	size_t n = 0, cap = 4096;
	float* v = (float*) malloc(cap * 3 * 8 * sizeof(float));
	#define PUT(x, y) do { float* p_ = v + (n * 3 + k_) * 8; p_[0] = (float) (x); p_[1] = (float) (y); p_[2] = 0.5f; \
		p_[3] = (float) rngU(rng); p_[4] = (float) rngU(rng); p_[5] = (float) rngU(rng); p_[6] = 0; p_[7] = 0; ++k_; } while (0)
	/* pixel-centre aligned fan: ndc = (px + 0.5) * 2 / W - 1 */
	double W = s->W, H = s->H;
	int cx = 64, cy = 96;
	for (int i = 0; i < 24 && n < cap; ++i, ++n) {
		int k_ = 0;
		double a0 = 2 * PI_D * i / 24, a1 = 2 * PI_D * (i + 1) / 24;
		int x0 = cx + (int) floor(40 * dcos(a0) + 0.5), y0 = cy + (int) floor(40 * dsin(a0) + 0.5);
		int x1 = cx + (int) floor(40 * dcos(a1) + 0.5), y1 = cy + (int) floor(40 * dsin(a1) + 0.5);
		PUT((cx + 0.5) * 2 / W - 1, 1 - (cy + 0.5) * 2 / H);
		PUT((x0 + 0.5) * 2 / W - 1, 1 - (y0 + 0.5) * 2 / H);
		PUT((x1 + 0.5) * 2 / W - 1, 1 - (y1 + 0.5) * 2 / H);
	}
	/* grid of axis-aligned quads on integer pixel edges and centres */
	for (int gy = 0; gy < 6; ++gy)
		for (int gx = 0; gx < 8 && n + 2 < cap; ++gx) {
			double off = (gx + gy) & 1 ? 0.5 : 0.0;
			double x0 = 130 + gx * 14 + off, y0 = 10 + gy * 14 + off, x1 = x0 + 14, y1 = y0 + 14;
			double X0 = x0 * 2 / W - 1, X1 = x1 * 2 / W - 1, Y0 = 1 - y0 * 2 / H, Y1 = 1 - y1 * 2 / H;
			int k_ = 0; PUT(X0, Y0); PUT(X1, Y1); PUT(X0, Y1); ++n;
			k_ = 0; PUT(X0, Y0); PUT(X1, Y0); PUT(X1, Y1); ++n;
		}
	/* slivers, tiny and degenerate triangles */
	for (int i = 0; i < 300 && n < cap; ++i, ++n) {
		int k_ = 0;
		double x = rngRange(rng, -0.9, 0.9), y = rngRange(rng, -0.9, -0.1);
		double sz = (i % 3 == 0) ? rngRange(rng, 0.001, 0.02) : rngRange(rng, 0.02, 0.3);
		if (i % 7 == 0) { PUT(x, y); PUT(x + sz, y + sz); PUT(x + 2 * sz, y + 2 * sz); }
		else if (i % 5 == 0) { PUT(x, y); PUT(x + sz, y + 0.002); PUT(x + 2 * sz, y); }
		else { PUT(x, y); PUT(x + rngRange(rng, -sz, sz), y + sz); PUT(x + sz, y + rngRange(rng, -sz, sz)); }
	}
	#undef PUT
	s->nTris = n;
	addVB(s, v, 32, n * 3 * 32);
	free(v);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->passOffset = 3; u->passCount = 3;
	}
	s->uni[1].model = mat4ConstructTranslate(0.013f, -0.37f, 0.f);
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_AFFINE) };
	program(s, 0, srpVsTransform, srpFsPrimitiveId, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	s->depthInit = 1.0f;
	s->render = renderRules;
	s->draws = 2;
}

static void renderScissor(Scene* s, SRPFramebuffer* fb)
{
	srpScissorTest(true);
	srpScissorOptions(40, 30, 150, 100);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, 3 * s->nTris);
	srpScissorOptions(200, 150, 100, 100);   /* partly outside the framebuffer */
	drawV(s, 0, fb, 1, SRP_PRIM_LINES, 0, 3 * s->nTris - (3 * s->nTris) % 2);
	srpScissorTest(false);
	srpRasterPointSize(2.f);
	drawV(s, 0, fb, 1, SRP_PRIM_POINTS, 0, 3 * s->nTris);
}

static void buildScissor(Scene* s, Rng* rng)
{
	featureSize(s);
	s->nTris = 60;
	float* v = (float*) malloc(s->nTris * 3 * 8 * sizeof(float));
	randomTris(rng, v, s->nTris, 2.0, 2.0, 8.0, 8);
	addVB(s, v, 32, s->nTris * 3 * 32);
	free(v);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 20.f);
		u->passOffset = 3; u->passCount = 3;
	}
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsPrimitiveId, 0, 1, v0);
	s->depthInit = 1.0f;
	s->render = renderScissor;
	s->draws = 3;
}

static void renderStencil(Scene* s, SRPFramebuffer* fb)
{
	const size_t n = 3 * s->nTris;
	srpRasterCullFace(SRP_FACE_NONE);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	srpStencilTest(true);
	/* pass 1: replace with 1 where drawn, different ops for back faces */
	srpStencilFunc(SRP_COMPARE_ALWAYS, 1, 0xFF);
	srpStencilOpSeparate(SRP_FACE_FRONT, SRP_STENCIL_KEEP, SRP_STENCIL_INCR_WRAP, SRP_STENCIL_REPLACE);
	srpStencilOpSeparate(SRP_FACE_BACK, SRP_STENCIL_KEEP, SRP_STENCIL_DECR_WRAP, SRP_STENCIL_INVERT);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, n);
	/* pass 2: outline where stencil != 1, no depth test, write-masked ops */
	srpStencilFuncSeparate(SRP_FACE_FRONT_AND_BACK, SRP_COMPARE_NOTEQUAL, 1, 0xFF);
	srpStencilOp(SRP_STENCIL_INCR, SRP_STENCIL_DECR, SRP_STENCIL_ZERO);
	srpStencilWriteMaskSeparate(SRP_FACE_BACK, 0x0F);
	srpDepthTest(false);
	drawV(s, 0, fb, 1, SRP_PRIM_TRIANGLES, 0, n);
	/* pass 3: every compare op on its own slice */
	srpDepthTest(true);
	srpStencilWriteMask(0xFF);
	for (int op = 0; op < 8; ++op) {
		srpStencilFunc((SRPCompareOp) op, (uint8_t) (op * 37), (uint8_t) (0xF0 | op));
		srpStencilOp((SRPStencilOp) op, (SRPStencilOp) ((op + 3) & 7), (SRPStencilOp) ((op + 5) & 7));
		size_t first = (size_t) op * (s->nTris / 8) * 3;
		drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, first, 3 * (s->nTris / 8));
	}
}

static void buildStencil(Scene* s, Rng* rng)
{
	featureSize(s);
	s->nTris = 96;
	float* v = (float*) malloc(s->nTris * 3 * 8 * sizeof(float));
	randomTris(rng, v, s->nTris, 1.5, 2.0, 7.0, 8);
	addVB(s, v, 32, s->nTris * 3 * 32);
	free(v);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 20.f);
		u->passOffset = 3; u->passCount = 3;
		u->color[0] = 1; u->color[1] = 0.2f; u->color[2] = 0.1f;
	}
	s->uni[1].model = mat4ConstructScale(1.05f, 1.05f, 1.05f);
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsSolid, 0, 1, v0);
	s->depthInit = 1.0f;
	s->stencilInit = 3;
	s->usesStencil = 1;
	s->render = renderStencil;
	s->draws = 10;
}

static void renderPolyModes(Scene* s, SRPFramebuffer* fb)
{
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	srpRasterCullFace(SRP_FACE_BACK);
	srpRasterPolygonMode(SRP_POLYGON_MODE_LINE);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
	srpRasterPolygonMode(SRP_POLYGON_MODE_POINT);
	srpRasterPointSize(2.f);
	drawI(s, 0, 1, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
	srpRasterPolygonMode(SRP_POLYGON_MODE_FILL);
	srpRasterCullFace(SRP_FACE_FRONT_AND_BACK);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);  /* draws nothing */
}

/* Polygon modes LINE and POINT on a sphere that crosses the near plane. */
static void buildPolyModes(Scene* s, Rng* rng)
{
	featureSize(s);
	Mesh m = uvSphere(10, 20, rng, 1.0f);
	addVB(s, m.v, m.stride * 4, m.nv * m.stride * 4);
	for (size_t i = 0; i < m.nv; ++i) m.v[i * m.stride + 2] += 0.35f;
	addVB(s, m.v, m.stride * 4, m.nv * m.stride * 4);
	addIB(s, SRP_UINT32, m.idx, m.ni * 4);
	s->nTris = 2 * m.ni / 3;
	freeMesh(&m);
	SRPStdUniform* u = &s->uni[0];
	baseUniform(u);
	u->model = rotation(0.3, 0.7, 0.1);
	u->view = mat4ConstructTranslate(0.2f, 0, 1.4f);
	u->projection = perspective60((float) s->W / (float) s->H, 0.6f, 30.f);
	u->passOffset = 8; u->passCount = 3;
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsPrimitiveId, 0, 1, v0);
	s->depthInit = 1.0f;
	s->render = renderPolyModes;
	s->draws = 3;
}

static void renderTopologies(Scene* s, SRPFramebuffer* fb)
{
	srpRasterCullFace(SRP_FACE_BACK);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LEQUAL);
	size_t n = s->vbytes[0] / 32;
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLE_STRIP, 0, n / 2);
	drawV(s, 0, fb, 1, SRP_PRIM_TRIANGLE_FAN, n / 2, n / 4);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 1, 3 * 20 + 2);  /* count % 3 != 0 warns */
	drawI(s, 1, 0, fb, 1, SRP_PRIM_TRIANGLE_STRIP, 0, 40);
	drawV(s, 0, fb, 1, SRP_PRIM_LINE_STRIP, 3 * n / 4, n / 8);
	drawV(s, 0, fb, 0, SRP_PRIM_LINE_LOOP, 7 * n / 8, n / 8);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_LINES, 5, 31);               /* odd count warns */
	drawV(s, 0, fb, 1, SRP_PRIM_POINTS, 0, n);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, n - 2, 9);          /* out of range: error, no-op */
}

/* Every topology, u8 and u32 indices, non-indexed draws, the excess-vertex
 * warnings and an out-of-range draw that must be rejected. */
static void buildTopologies(Scene* s, Rng* rng)
{
	featureSize(s);
	size_t n = 256;
	float* v = (float*) malloc(n * 8 * sizeof(float));
	for (size_t i = 0; i < n; ++i) {
		float* p = v + 8 * i;
		double a = 2 * PI_D * (double) i / 37.0;
		double r = 0.3 + 0.7 * rngU(rng);
		p[0] = (float) (r * dcos(a) * 2.5); p[1] = (float) (r * dsin(a) * 1.8); p[2] = (float) rngRange(rng, 3, 6);
		p[3] = (float) rngU(rng); p[4] = (float) rngU(rng); p[5] = (float) rngU(rng); p[6] = 0; p[7] = 0;
	}
	addVB(s, v, 32, n * 32);
	free(v);
	uint8_t i8[200];
	for (int i = 0; i < 200; ++i) i8[i] = (uint8_t) ((i * 13 + 5) % 256);
	addIB(s, SRP_UINT8, i8, sizeof i8);
	uint32_t i32[64];
	for (int i = 0; i < 64; ++i) i32[i] = (uint32_t) ((i * 29 + 3) % 256);
	addIB(s, SRP_UINT32, i32, sizeof i32);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 20.f);
		u->passOffset = 3; u->passCount = 3;
	}
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsPrimitiveId, 0, 1, v0);
	s->depthInit = 1.0f;
	s->render = renderTopologies;
	s->draws = 9;
}

static void renderLateZ(Scene* s, SRPFramebuffer* fb)
{
	srpRasterCullFace(SRP_FACE_NONE);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, 3 * s->nTris / 2);
	srpStencilTest(true);
	srpStencilOp(SRP_STENCIL_INCR, SRP_STENCIL_INVERT, SRP_STENCIL_INCR_WRAP);
	drawV(s, 0, fb, 1, SRP_PRIM_TRIANGLES, 3 * s->nTris / 2, 3 * s->nTris / 2);
	drawV(s, 0, fb, 1, SRP_PRIM_LINES, 0, 3 * s->nTris / 2);
}

/* A fragment shader that writes fragDepth (late depth test, in-order shading)
 * mixed with ordinary early-depth draws. */
static void buildLateZ(Scene* s, Rng* rng)
{
	featureSize(s);
	s->nTris = 64;
	float* v = (float*) malloc(s->nTris * 3 * 8 * sizeof(float));
	randomTris(rng, v, s->nTris, 1.5, 2.0, 7.0, 8);
	addVB(s, v, 32, s->nTris * 3 * 32);
	free(v);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 20.f);
		u->passOffset = 3; u->passCount = 3;
		u->depthScale = 0.75f; u->depthBias = 0.01f;
	}
	SRPVaryingInfo v0[1] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsTransform, srpFsVaryingColor, 0, 1, v0);
	program(s, 1, srpVsTransform, srpFsDepthOverwrite, 1, 1, v0);
	s->depthInit = 1.0f;
	s->usesStencil = 1;
	s->render = renderLateZ;
	s->draws = 3;
}

static void renderLit(Scene* s, SRPFramebuffer* fb)
{
	srpRasterCullFace(SRP_FACE_BACK);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
	drawI(s, 0, 1, fb, 1, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
}

/* Lighting shaders (textured Blinn-Phong, marble) on world-space varyings. */
static void buildLit(Scene* s, Rng* rng)
{
	featureSize(s);
	Mesh m = uvSphere(24, 48, rng, 0.8f);
	for (size_t i = 0; i < m.nv; ++i) m.v[i * m.stride] -= 0.9f;
	addVB(s, m.v, m.stride * 4, m.nv * m.stride * 4);
	for (size_t i = 0; i < m.nv; ++i) m.v[i * m.stride] += 1.8f;
	addVB(s, m.v, m.stride * 4, m.nv * m.stride * 4);
	addIB(s, SRP_UINT32, m.idx, m.ni * 4);
	s->nTris = 2 * m.ni / 3;
	freeMesh(&m);
	uint8_t* tex = (uint8_t*) malloc(32 * 32 * 3);
	for (int i = 0; i < 32 * 32 * 3; ++i) tex[i] = (uint8_t) (rngNext(rng) >> 56);
	s->tex = makeTexture(s, tex, 32, 32, TW_REPEAT, TW_REPEAT);
	free(tex);
	for (int k = 0; k < 2; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->view = mat4ConstructTranslate(0, 0, 3.2f);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 20.f);
		u->normalOffset = 3; u->uvOffset = 6;
		u->cameraPos[2] = -3.2f;
		u->texture = k == 0 ? s->tex : NULL;
		u->nLights = k == 0 ? 1 : 16;
		for (int l = 0; l < 16; ++l) {
			u->lightPos[l][0] = (float) rngRange(rng, -4, 4);
			u->lightPos[l][1] = (float) rngRange(rng, -4, 4);
			u->lightPos[l][2] = (float) rngRange(rng, -5, 0);
			for (int c = 0; c < 3; ++c) u->lightColor[l][c] = (float) rngRange(rng, 0.1, k == 0 ? 1.0 : 0.3);
		}
	}
	SRPVaryingInfo v0[3] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsWorld, srpFsBlinnPhong, 0, 3, v0);
	program(s, 1, srpVsWorld, srpFsMarble, 0, 3, v0);
	s->depthInit = 1.0f;
	s->render = renderLit;
	s->draws = 2;
}

/* The learned-shading workload: the soup's geometry (random geodesic
 * spheres, about 20% of them cut by the near plane), triangles only, shaded
 * by the expensive procedural shader -- 8-octave value-noise marble lit by
 * 16 point lights (Blinn-Phong, shininess 64). The lights and the marble
 * belong to the material, which every seed shares; the seed only places the
 * spheres. */
static void renderMSoup(Scene* s, SRPFramebuffer* fb)
{
	srpRasterFrontFace(SRP_WINDING_CCW);
	srpRasterCullFace(SRP_FACE_BACK);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
}

static void buildMSoup(Scene* s, Rng* rng)
{
	s->W = 1920; s->H = 1080;
	if (s->scale < 1.0) {
		const double lin = dexp(0.5 * dlog(s->scale));
		s->W = (int) (1920 * lin) & ~7; s->H = (int) (1080 * lin) & ~7;
		if (s->W < 64) s->W = 64;
		if (s->H < 48) s->H = 48;
	}
	const size_t target = (size_t) (2000000 * s->scale);
	float* verts = NULL; uint32_t* idx = NULL;
	size_t nv = 0, ni = 0, capv = 0, capi = 0;
	uint32_t meshId = 0;
	while (ni / 3 < target) {
		double tris = logUniform(rng, 5000, 50000);
		int f = (int) floor(sqrt(tris / 20) + 0.5);
		double r = logUniform(rng, 0.05, 2.0);
		double c[3];
		if (rngU(rng) < 0.2) {
			double zc = 0.1 + r * rngRange(rng, -0.5, 0.5);
			double rho = sqrt(fmax(0.0, 1.2 * r * r - zc * zc)) + r * rngRange(rng, 0.0, 0.4);
			double ang = rngRange(rng, 0, 2 * PI_D);
			c[0] = rho * dcos(ang); c[1] = rho * dsin(ang); c[2] = zc;
		} else {
			c[0] = rngRange(rng, -10, 10); c[1] = rngRange(rng, -10, 10); c[2] = rngRange(rng, 0.5, 20.5);
		}
		appendGeodesic(&verts, &nv, &capv, &idx, &ni, &capi, f, c, r, meshId++, rng);
	}
	addVB(s, verts, 48, nv * 48);
	addIB(s, SRP_UINT32, idx, ni * 4);
	s->nTris = ni / 3;
	free(verts); free(idx);
	SRPStdUniform* u = &s->uni[0];
	baseUniform(u);
	u->projection = perspective60((float) s->W / (float) s->H, 0.1f, 100.f);
	u->normalOffset = 3; u->uvOffset = 6;
	u->nLights = 16;
	Rng mat = { 0x5EED0F11A7E51A1Dull };   /* the material: the same for every seed */
	for (int l = 0; l < 16; ++l) {
		u->lightPos[l][0] = (float) rngRange(&mat, -12, 12);
		u->lightPos[l][1] = (float) rngRange(&mat, -12, 12);
		u->lightPos[l][2] = (float) rngRange(&mat, -2, 18);
		for (int k = 0; k < 3; ++k) u->lightColor[l][k] = (float) rngRange(&mat, 0.1, 0.5);
	}
	SRPVaryingInfo v0[3] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsWorld, srpFsMarble, 0, 3, v0);
	s->depthInit = 1.0f;
	s->render = renderMSoup;
	s->draws = 1;
}

/* The marble soup with the marble's noise cut to its first octave: the
 * same geometry, camera and lights for a given seed, shaded by the cheap
 * level of detail of the same procedural shader. The baseline that the
 * learned stand-in of the 8-octave shader is measured against. */
static void buildMSoupLod(Scene* s, Rng* rng)
{
	buildMSoup(s, rng);
	s->uni[0].marbleOctaves = 1;
}

/* One scene of the batched workload: a single mesh of random triangles
 * (log-uniform 12 to 200k of them) in its own framebuffer (each side
 * log-uniform 64 to 1024), random camera, textured Blinn-Phong with one
 * light. The mesh is a randomly displaced grid, so its triangles are small
 * and connected; its placement makes some scenes cross the near plane.
 * State: CCW front faces, back-face culling, depth LESS, depth cleared to 1. */
static void bsceneState(void)
{
	srpRasterFrontFace(SRP_WINDING_CCW);
	srpRasterCullFace(SRP_FACE_BACK);
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
}

static void renderBScene(Scene* s, SRPFramebuffer* fb)
{
	bsceneState();
	drawI(s, 0, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, s->ibytes[0] / 4);
}

static void buildBScene(Scene* s, Rng* rng)
{
	double w = logUniform(rng, 64, 1024), h = logUniform(rng, 64, 1024);
	double tris = logUniform(rng, 12, 200000);
	if (s->scale < 1.0) {
		const double lin = dexp(0.5 * dlog(s->scale));
		w *= lin; h *= lin; tris *= s->scale;
	}
	s->W = (int) w < 16 ? 16 : (int) w;
	s->H = (int) h < 16 ? 16 : (int) h;
	if (tris < 12) tris = 12;
	/* grid of gx x gy cells, two triangles per cell */
	const double aspect = rngRange(rng, 0.5, 2.0);
	int gx = (int) (dexp(0.5 * dlog(tris / 2 * aspect)) + 0.5);
	if (gx < 2) gx = 2;
	int gy = (int) (tris / 2 / gx + 0.5);
	if (gy < 2) gy = 2;
	const size_t nv = (size_t) (gx + 1) * (gy + 1), words = 8;
	float* v = (float*) malloc(nv * words * sizeof(float));
	const double bump = rngRange(rng, 0.0, 0.08);
	for (int j = 0; j <= gy; ++j)
		for (int i = 0; i <= gx; ++i) {
			float* p = v + ((size_t) j * (gx + 1) + i) * words;
			const double u = (double) i / gx, t = (double) j / gy;
			const double dz = rngRange(rng, -bump, bump);
			p[0] = (float) ((u - 0.5) * 2.0 * aspect / (aspect > 1 ? aspect : 1));
			p[1] = (float) ((t - 0.5) * 2.0 / (aspect > 1 ? aspect : 1));
			p[2] = (float) dz;
			const double nx = rngRange(rng, -0.3, 0.3), ny = rngRange(rng, -0.3, 0.3);
			p[3] = (float) nx; p[4] = (float) ny; p[5] = 1.0f;
			p[6] = (float) (u * 4.0); p[7] = (float) (t * 4.0);
		}
	const size_t ni = (size_t) gx * gy * 6;
	uint32_t* idx = (uint32_t*) malloc(ni * sizeof(uint32_t));
	size_t k = 0;
	for (int j = 0; j < gy; ++j)
		for (int i = 0; i < gx; ++i) {
			const uint32_t a = (uint32_t) (j * (gx + 1) + i), b = a + 1, c = a + (uint32_t) (gx + 1), d = c + 1;
			idx[k++] = a; idx[k++] = b; idx[k++] = d;
			idx[k++] = a; idx[k++] = d; idx[k++] = c;
		}
	addVB(s, v, words * 4, nv * words * 4);
	addIB(s, SRP_UINT32, idx, ni * 4);
	s->nTris = ni / 3;
	free(v);
	free(idx);
	uint8_t* tex = (uint8_t*) malloc(64 * 64 * 3);
	for (int i = 0; i < 64 * 64 * 3; ++i) tex[i] = (uint8_t) (rngNext(rng) >> 56);
	s->tex = makeTexture(s, tex, 64, 64, TW_REPEAT, TW_REPEAT);
	free(tex);
	SRPStdUniform* u = &s->uni[0];
	baseUniform(u);
	/* tilted by up to about 70 degrees, so the front side mostly faces the camera */
	double ang[3];
	ang[0] = rngRange(rng, -1.2, 1.2);
	ang[1] = rngRange(rng, -1.2, 1.2);
	ang[2] = rngRange(rng, 0, 2 * PI_D);
	u->model = rotation(ang[0], ang[1], ang[2]);
	const double dist = rngRange(rng, 0.9, 3.5);
	u->view = mat4ConstructTranslate(0, 0, (float) dist);
	u->projection = perspective60((float) s->W / (float) s->H, 0.1f, 100.f);
	u->cameraPos[2] = (float) -dist;
	u->normalOffset = 3; u->uvOffset = 6;
	u->texture = s->tex;
	u->nLights = 1;
	u->lightPos[0][0] = (float) rngRange(rng, -3, 3);
	u->lightPos[0][1] = (float) rngRange(rng, -3, 3);
	u->lightPos[0][2] = (float) rngRange(rng, -4, -1);
	for (int c = 0; c < 3; ++c) u->lightColor[0][c] = (float) rngRange(rng, 0.5, 1.0);
	SRPVaryingInfo v0[3] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsWorld, srpFsBlinnPhong, 0, 3, v0);
	s->depthInit = 1.0f;
	s->render = renderBScene;
	s->draws = 1;
}

/* The batched learned-shading workload: a batched-workload scene shaded by
 * the expensive marble shader with 16 point lights. The lights belong to the
 * material, which every seed shares. */
static void buildBMScene(Scene* s, Rng* rng)
{
	buildBScene(s, rng);
	SRPStdUniform* u = &s->uni[0];
	u->texture = NULL;
	u->nLights = 16;
	Rng mat = { 0xB1A5ED0F1A7E51A1ull };
	for (int l = 0; l < 16; ++l) {
		u->lightPos[l][0] = (float) rngRange(&mat, -4, 4);
		u->lightPos[l][1] = (float) rngRange(&mat, -4, 4);
		u->lightPos[l][2] = (float) rngRange(&mat, -6, 1);
		for (int k = 0; k < 3; ++k) u->lightColor[l][k] = (float) rngRange(&mat, 0.1, 0.5);
	}
	SRPVaryingInfo v0[3] = { vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE),
	                         vi(2, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE) };
	program(s, 0, srpVsWorld, srpFsMarble, 0, 3, v0);
}

/* ------------------------------------------------- packed varying layouts */

#define PACK13_BYTES 13   /* position (12 B) + uint8 palette index */
#define PACK49_BYTES (12 + SRP_MIXED_BLOCK_BYTES)

static void renderVaryings(Scene* s, SRPFramebuffer* fb)
{
	const size_t half = s->param[0], nTri = s->param[1];
	srpDepthTest(true);
	srpDepthCompareOp(SRP_COMPARE_LESS);
	srpRasterCullFace(SRP_FACE_NONE);
	/* 13-byte vertices, one uint8 flat varying: first, then last provoking vertex */
	srpProvokingVertexMode(SRP_PROVOKING_VERTEX_FIRST);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 0, 3 * half);
	srpProvokingVertexMode(SRP_PROVOKING_VERTEX_LAST);
	drawV(s, 0, fb, 0, SRP_PRIM_TRIANGLES, 3 * half, 3 * half);
	/* 49-byte vertices, the 37-byte mixed block: perspective, affine, flat */
	const size_t third = nTri / 3;
	drawI(s, 0, 1, fb, 1, SRP_PRIM_TRIANGLES, 0, 3 * third);
	srpProvokingVertexMode(SRP_PROVOKING_VERTEX_FIRST);
	drawI(s, 0, 1, fb, 2, SRP_PRIM_TRIANGLES, 3 * third, 3 * third);
	srpProvokingVertexMode(SRP_PROVOKING_VERTEX_LAST);
	drawI(s, 0, 1, fb, 3, SRP_PRIM_TRIANGLES, 6 * third, 3 * (nTri - 2 * third));
	/* the same block on lines (two-vertex interpolation) and points (raw) */
	srpDepthCompareOp(SRP_COMPARE_LEQUAL);
	drawI(s, 0, 1, fb, 4, SRP_PRIM_LINE_STRIP, 0, 3 * third);
	srpRasterPointSize(3.f);
	drawV(s, 1, fb, 5, SRP_PRIM_POINTS, 0, 3 * nTri);
}

static void packMixed(Rng* rng, unsigned char* blk)
{
	int8_t a = (int8_t) (rngNext(rng) >> 56);
	double d[2] = { rngRange(rng, -4, 4), rngRange(rng, -3, 3) };
	uint16_t b = (uint16_t) (rngNext(rng) >> 48);
	float f[2] = { (float) rngRange(rng, -2, 2), (float) rngRange(rng, -2, 2) };
	int16_t c = (int16_t) (rngNext(rng) >> 48);
	uint64_t e = rngNext(rng);
	memcpy(blk, &a, 1); memcpy(blk + 1, d, 16); memcpy(blk + 17, &b, 2);
	memcpy(blk + 19, f, 8); memcpy(blk + 27, &c, 2); memcpy(blk + 29, &e, 8);
}

/* Every varying element type the reference interpolates
 * (src/pipeline/interpolation.c:63-163) in byte-packed layouts:
 * - 13-byte vertices (position + a uint8, as in the reference's own flat
 *   interpolation test scene, tests/scenes/interpolation/flat.c:8-17), the
 *   uint8 declared as one UINT8 flat varying, with both provoking vertices;
 * - 49-byte vertices whose 37-byte varying block holds int8, 2 doubles,
 *   uint16, 2 floats, int16 and uint64 at odd offsets, drawn with every
 *   floating attribute perspective, affine and flat, then as a line strip and
 *   as points. Triangles straddle the near plane, so clipping interpolates the
 *   doubles and copies the integers from the pair's provoking vertex. */
static void buildVaryings(Scene* s, Rng* rng)
{
	featureSize(s);
	const double sc = s->scale < 1 ? s->scale : 1;
	const size_t nTri0 = (size_t) (120 * sc) + 8, nTri = (size_t) (240 * sc) + 12;
	s->param[0] = (int) (nTri0 / 2);
	s->param[1] = (int) nTri;
	float* tmp = (float*) malloc(nTri * 3 * 8 * sizeof(float));
	/* 13-byte vertices */
	randomTris(rng, tmp, nTri0, 3.0, 0.2, 11.0, 8);
	unsigned char* v13 = (unsigned char*) malloc(nTri0 * 3 * PACK13_BYTES);
	for (size_t i = 0; i < nTri0 * 3; ++i) {
		memcpy(v13 + i * PACK13_BYTES, tmp + i * 8, 12);
		v13[i * PACK13_BYTES + 12] = (unsigned char) (i % 5 == 4 ? (rngNext(rng) >> 56) : (rngNext(rng) % 3));
	}
	addVB(s, v13, PACK13_BYTES, nTri0 * 3 * PACK13_BYTES);
	free(v13);
	/* 49-byte vertices */
	randomTris(rng, tmp, nTri, 3.0, -1.0, 12.0, 8);
	unsigned char* v49 = (unsigned char*) malloc(nTri * 3 * PACK49_BYTES);
	for (size_t i = 0; i < nTri * 3; ++i) {
		memcpy(v49 + i * PACK49_BYTES, tmp + i * 8, 12);
		packMixed(rng, v49 + i * PACK49_BYTES + 12);
	}
	addVB(s, v49, PACK49_BYTES, nTri * 3 * PACK49_BYTES);
	free(v49);
	free(tmp);
	const size_t nv = nTri * 3;
	uint16_t* idx = (uint16_t*) malloc(nv * sizeof(uint16_t));
	for (size_t i = 0; i < nv; ++i) idx[i] = (uint16_t) ((i * 7919) % nv);
	addIB(s, SRP_UINT16, idx, nv * 2);
	free(idx);
	for (int k = 0; k < 6; ++k) {
		SRPStdUniform* u = &s->uni[k];
		baseUniform(u);
		u->model = rotation(0.05 * k, 0.1, 0.02);
		u->projection = perspective60((float) s->W / (float) s->H, 0.5f, 12.f);
		u->passOffset = 12;
		u->passCount = k == 0 ? 1 : SRP_MIXED_BLOCK_BYTES;
	}
	SRPVaryingInfo v8[1] = { vi(1, SRP_UINT8, SRP_INTERPOLATION_MODE_FLAT) };
	program(s, 0, srpVsBytes, srpFsBytePalette, 0, 1, v8);
	const SRPInterpolationMode modes[5] = { SRP_INTERPOLATION_MODE_PERSPECTIVE, SRP_INTERPOLATION_MODE_AFFINE,
	                                        SRP_INTERPOLATION_MODE_FLAT, SRP_INTERPOLATION_MODE_PERSPECTIVE,
	                                        SRP_INTERPOLATION_MODE_AFFINE };
	for (int k = 0; k < 5; ++k) {
		const SRPInterpolationMode m = modes[k];
		/* integer members are flat whatever mode they are given */
		SRPVaryingInfo mix[6] = { vi(1, SRP_INT8, m), vi(2, SRP_DOUBLE, m), vi(1, SRP_UINT16, m),
		                          vi(2, SRP_FLOAT, m), vi(1, SRP_INT16, m), vi(1, SRP_UINT64, m) };
		program(s, 1 + k, srpVsBytes, srpFsMixed, 0, 6, mix);
	}
	s->nTris = nTri0 + nTri;
	s->nLines = 3 * (nTri / 3) - 1;
	s->nPoints = 3 * nTri;
	s->depthInit = 1.0f;
	s->render = renderVaryings;
	s->draws = 7;
}

/* ------------------------------------------------------------- registry */

typedef struct SceneDef { const char* name; void (*build)(Scene*, Rng*); } SceneDef;

static const SceneDef DEFS[] = {
	{ "sphere", buildSphere },
	{ "soup", buildSoup },
	{ "clip_tris", buildClipTris },
	{ "clip_lines", buildClipLines },
	{ "points", buildPoints },
	{ "interp", buildInterp },
#ifndef SCENES_REF
	{ "texfilter", buildTexFilter },
#endif
	{ "depth_ops", buildDepthOps },
	{ "raster_rules", buildRules },
	{ "scissor", buildScissor },
	{ "stencil", buildStencil },
	{ "poly_modes", buildPolyModes },
	{ "topologies", buildTopologies },
	{ "late_z", buildLateZ },
	{ "lit", buildLit },
	{ "varyings", buildVaryings },
	{ "bscene", buildBScene },
	{ "msoup", buildMSoup },
	{ "msoup_lod", buildMSoupLod },
	{ "bmscene", buildBMScene },
};

const char* const* sceneNames(void)
{
	static const char* names[sizeof DEFS / sizeof DEFS[0] + 1];
	for (size_t i = 0; i < sizeof DEFS / sizeof DEFS[0]; ++i) names[i] = DEFS[i].name;
	names[sizeof DEFS / sizeof DEFS[0]] = NULL;
	return names;
}

Scene* sceneCreate(const char* name, uint64_t seed, double scale)
{
	for (size_t i = 0; i < sizeof DEFS / sizeof DEFS[0]; ++i) {
		if (strcmp(DEFS[i].name, name) != 0) continue;
		Scene* s = (Scene*) calloc(1, sizeof(Scene));
		snprintf(s->name, sizeof s->name, "%s", name);
		s->seed = seed;
		s->scale = scale > 0 && scale < 1 ? scale : 1.0;
		s->hash = 0xCBF29CE484222325ull;
		Rng rng = { seed * 0x9E3779B97F4A7C15ull + 0x1234567ull };
		DEFS[i].build(s, &rng);
		hashUniforms(s);
		return s;
	}
	return NULL;
}

void sceneDestroy(Scene* s)
{
	if (!s) return;
	for (int k = 0; k < s->nvb; ++k) { srpFreeVertexBuffer(s->vb[k]); hostFree(s->vdata[k]); }
	for (int k = 0; k < s->nib; ++k) { srpFreeIndexBuffer(s->ib[k]); hostFree(s->idata[k]); }
	if (s->tex) srpFreeTexture(s->tex);
	for (int k = 0; k < 2; ++k)
		if (s->texExtra[k]) srpFreeTexture(s->texExtra[k]);
	free(s);
}

void sceneGetInfo(const Scene* s, SceneInfo* info)
{
	memset(info, 0, sizeof *info);
	info->width = s->W; info->height = s->H;
	info->inputTriangles = s->nTris; info->inputLines = s->nLines; info->inputPoints = s->nPoints;
	for (int k = 0; k < s->nvb; ++k) info->vertexBytes += s->vbytes[k];
	for (int k = 0; k < s->nib; ++k) info->indexBytes += s->ibytes[k];
	info->textureBytes = s->texBytes;
	info->draws = s->draws;
	info->usesStencil = s->usesStencil;
}

uint64_t sceneInputHash(const Scene* s) { return s->hash; }

int sceneDumpInputs(const Scene* s, const char* path)
{
	FILE* f = fopen(path, "wb");
	if (!f) return 1;
	for (int k = 0; k < s->nvb; ++k) fwrite(s->vdata[k], 1, s->vbytes[k], f);
	for (int k = 0; k < s->nib; ++k) fwrite(s->idata[k], 1, s->ibytes[k], f);
	for (int k = 0; k < s->nprog; ++k) fwrite(&s->uni[k], 1, offsetof(SRPStdUniform, texture), f);
	fclose(f);
	return 0;
}

void sceneUpload(Scene* s)
{
	for (int k = 0; k < s->nvb; ++k) srpVertexBufferCopyData(s->vb[k], s->vstride[k], s->vbytes[k], s->vdata[k]);
	for (int k = 0; k < s->nib; ++k) srpIndexBufferCopyData(s->ib[k], s->itype[k], s->ibytes[k], s->idata[k]);
}

void scenePrepareFramebuffer(Scene* s, SRPFramebuffer* fb)
{
	srpFramebufferClear(fb);
#ifdef SCENES_GPU
	srpGpuFramebufferFill(fb, 0, s->depthInit, s->stencilInit, SRP_GPU_FILL_DEPTH | SRP_GPU_FILL_STENCIL);
	if (srpGpuGetFramebufferMode() == SRP_GPU_FB_COHERENT) srpGpuFramebufferSync(fb);
#else
	for (size_t i = 0; i < fb->size; ++i) { fb->depth[i] = s->depthInit; fb->stencil[i] = s->stencilInit; }
#endif
}

static void resetContext(void)
{
	SRPMessageCallback cb = srpContext.messageCallback;
	srpNewContext(&srpContext);
	srpContext.messageCallback = cb;
}

void sceneRender(Scene* s, SRPFramebuffer* fb)
{
	resetContext();
	s->render(s, fb);
}

#ifdef SCENES_GPU
int sceneDrawDesc(Scene* s, SRPFramebuffer* fb, SRPGpuDraw* out)
{
	if (s->render != renderBScene) return 1;
	out->indexBuffer = s->ib[0];
	out->vertexBuffer = s->vb[0];
	out->framebuffer = fb;
	out->program = &s->sp[0];
	out->primitive = SRP_PRIM_TRIANGLES;
	out->startIndex = 0;
	out->count = s->ibytes[0] / 4;
	return 0;
}

void sceneBatchRender(Scene** scenes, SRPFramebuffer** fbs, size_t n, SRPGpuDraw* scratch)
{
	resetContext();
	bsceneState();
	for (size_t i = 0; i < n; ++i) sceneDrawDesc(scenes[i], fbs[i], &scratch[i]);
	srpGpuDrawBatch(scratch, n);
}

void sceneUploadAsync(Scene* s)
{
	/* the first draw's buffers first (vertex, then index buffer), so that its
	 * vertex stage can start while the rest is still on the way */
	for (int k = 0; k < s->nvb; ++k) {
		srpGpuVertexBufferCopyDataAsync(s->vb[k], s->vstride[k], s->vbytes[k], s->vdata[k]);
		if (k == 0 && s->nib > 0) srpGpuIndexBufferCopyDataAsync(s->ib[0], s->itype[0], s->ibytes[0], s->idata[0]);
	}
	for (int k = 1; k < s->nib; ++k) srpGpuIndexBufferCopyDataAsync(s->ib[k], s->itype[k], s->ibytes[k], s->idata[k]);
	if (s->nvb == 0 && s->nib > 0) srpGpuIndexBufferCopyDataAsync(s->ib[0], s->itype[0], s->ibytes[0], s->idata[0]);
}

void sceneUploadBatchAsync(Scene** scenes, size_t n)
{
	size_t cap = 0;
	for (size_t i = 0; i < n; ++i) cap += (size_t) (scenes[i]->nvb > scenes[i]->nib ? scenes[i]->nvb : scenes[i]->nib);
	if (!cap) return;
	SRPVertexBuffer** vb = (SRPVertexBuffer**) malloc(cap * sizeof *vb);
	SRPIndexBuffer** ib = (SRPIndexBuffer**) malloc(cap * sizeof *ib);
	size_t* stride = (size_t*) malloc(cap * sizeof *stride);
	size_t* vbytes = (size_t*) malloc(cap * sizeof *vbytes);
	size_t* ibytes = (size_t*) malloc(cap * sizeof *ibytes);
	SRPType* itype = (SRPType*) malloc(cap * sizeof *itype);
	const void** vsrc = (const void**) malloc(cap * sizeof *vsrc);
	const void** isrc = (const void**) malloc(cap * sizeof *isrc);
	for (size_t first = 0; first < n; first += 256) {
		const size_t last = first + 256 < n ? first + 256 : n;
		size_t nv = 0, ni = 0;
		for (size_t i = first; i < last; ++i) {
			const Scene* s = scenes[i];
			for (int k = 0; k < s->nvb; ++k) {
				vb[nv] = s->vb[k]; stride[nv] = s->vstride[k]; vbytes[nv] = s->vbytes[k]; vsrc[nv] = s->vdata[k];
				++nv;
			}
			for (int k = 0; k < s->nib; ++k) {
				ib[ni] = s->ib[k]; itype[ni] = s->itype[k]; ibytes[ni] = s->ibytes[k]; isrc[ni] = s->idata[k];
				++ni;
			}
		}
		srpGpuVertexBufferCopyDataBatchAsync(vb, stride, vbytes, vsrc, nv);
		srpGpuIndexBufferCopyDataBatchAsync(ib, itype, ibytes, isrc, ni);
	}
	free(vb); free(ib); free(stride); free(vbytes); free(ibytes); free(itype); free(vsrc); free(isrc);
}

void scenePrepareBatch(Scene** scenes, SRPFramebuffer** fbs, size_t n)
{
	if (!n) return;
	int same = 1;
	for (size_t i = 1; i < n; ++i)
		if (scenes[i]->depthInit != scenes[0]->depthInit || scenes[i]->stencilInit != scenes[0]->stencilInit) same = 0;
	if (!same) {
		for (size_t i = 0; i < n; ++i) scenePrepareFramebuffer(scenes[i], fbs[i]);
		return;
	}
	/* srpFramebufferClear (colour 0) followed by the scene's depth and stencil */
	srpGpuFramebufferFillBatch((const SRPFramebuffer* const*) fbs, n, 0u, scenes[0]->depthInit, scenes[0]->stencilInit,
	                           SRP_GPU_FILL_COLOR | SRP_GPU_FILL_DEPTH | SRP_GPU_FILL_STENCIL);
}

int sceneBatchAutotune(Scene** scenes, SRPFramebuffer** fbs, size_t n, SRPGpuDraw* scratch, int repeats,
                       SRPGpuTuning* best)
{
	resetContext();
	bsceneState();
	for (size_t i = 0; i < n; ++i) sceneDrawDesc(scenes[i], fbs[i], &scratch[i]);
	return srpGpuAutotune(scratch, n, repeats, best);
}
#endif

int sceneRunOnce(const char* name, uint64_t seed, double scale,
                 uint32_t* color, float* depth, uint8_t* stencil, int* width, int* height)
{
	Scene* s = sceneCreate(name, seed, scale);
	if (!s) return 1;
	SRPFramebuffer* fb = srpNewFramebuffer((size_t) s->W, (size_t) s->H);
	scenePrepareFramebuffer(s, fb);
	sceneRender(s, fb);
#ifdef SCENES_GPU
	srpGpuFramebufferSync(fb);
#endif
	if (width) *width = s->W;
	if (height) *height = s->H;
	if (color) memcpy(color, fb->color, fb->size * 4);
	if (depth) memcpy(depth, fb->depth, fb->size * 4);
	if (stencil) memcpy(stencil, fb->stencil, fb->size);
	srpFreeFramebuffer(fb);
	sceneDestroy(s);
	return 0;
}
