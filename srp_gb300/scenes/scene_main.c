/* Command-line scene runner, linked against the CPU oracle or against the
 * reference library built from source (it is the "user program" and so
 * defines the global srpContext, as srp requires).
 *
 *   scene_runner list
 *   scene_runner render <scene> <seed> <scale> <out.bin>
 *       writes "SRPD", width, height, input hash, fragment count, then the
 *       colour (u32), depth (f32) and stencil (u8) planes
 *   scene_runner time <scene> <seed> <scale> <frames>
 *       renders `frames` frames (buffers resident, framebuffer prepared
 *       outside the timed region) and prints one JSON line */
#define _POSIX_C_SOURCE 199309L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "scenes.h"

SRPContext srpContext;

#ifdef SCENES_PORT
extern size_t srpPortFragmentCount;
static uint64_t fragments(void) { return srpPortFragmentCount; }
#else
static uint64_t fragments(void) { return 0; }
#endif

static double now(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec + ts.tv_nsec * 1e-9;
}

int main(int argc, char** argv)
{
	if (argc >= 2 && !strcmp(argv[1], "list")) {
		for (const char* const* n = sceneNames(); *n; ++n) printf("%s\n", *n);
		return 0;
	}
	if (argc < 6) {
		fprintf(stderr, "usage: %s render|time <scene> <seed> <scale> <out|frames>\n", argv[0]);
		return 2;
	}
	srpNewContext(&srpContext);
	const char* name = argv[2];
	uint64_t seed = strtoull(argv[3], NULL, 10);
	double scale = atof(argv[4]);
	Scene* s = sceneCreate(name, seed, scale);
	if (!s) { fprintf(stderr, "unknown scene %s\n", name); return 2; }
	SceneInfo info;
	sceneGetInfo(s, &info);
	SRPFramebuffer* fb = srpNewFramebuffer((size_t) info.width, (size_t) info.height);
	if (!strcmp(argv[1], "inputs")) {
		sceneDumpInputs(s, argv[5]);
	} else if (!strcmp(argv[1], "render")) {
		scenePrepareFramebuffer(s, fb);
		uint64_t f0 = fragments();
		sceneRender(s, fb);
		uint64_t nf = fragments() - f0;
		FILE* f = fopen(argv[5], "wb");
		if (!f) return 1;
		uint32_t hdr[2] = { (uint32_t) info.width, (uint32_t) info.height };
		uint64_t h = sceneInputHash(s);
		fwrite("SRPD", 1, 4, f);
		fwrite(hdr, 4, 2, f);
		fwrite(&h, 8, 1, f);
		fwrite(&nf, 8, 1, f);
		fwrite(fb->color, 4, fb->size, f);
		fwrite(fb->depth, 4, fb->size, f);
		fwrite(fb->stencil, 1, fb->size, f);
		fclose(f);
	} else if (!strcmp(argv[1], "time")) {
		int frames = atoi(argv[5]);
		double total = 0, best = 1e30;
		uint64_t nf = 0;
		for (int i = 0; i < frames; ++i) {
			scenePrepareFramebuffer(s, fb);
			uint64_t f0 = fragments();
			double t0 = now();
			sceneRender(s, fb);
			double dt = now() - t0;
			nf = fragments() - f0;
			total += dt;
			if (dt < best) best = dt;
		}
		printf("{\"scene\": \"%s\", \"frames\": %d, \"mean_s\": %.6f, \"best_s\": %.6f, \"fragments\": %llu, "
		       "\"triangles\": %zu, \"lines\": %zu, \"points\": %zu, \"width\": %d, \"height\": %d}\n",
		       name, frames, total / (frames > 0 ? frames : 1), best, (unsigned long long) nf,
		       info.inputTriangles, info.inputLines, info.inputPoints, info.width, info.height);
	}
	srpFreeFramebuffer(fb);
	sceneDestroy(s);
	return 0;
}
