/* Dumps the two input assets of the reference's own image tests
 * (tests/scenes/**), as the reference itself loads them, for
 * tests/golden/make_refimages.py. Test infrastructure: linked against the
 * reference's OBJ loader (examples/utility/objparser.c) and its copy of
 * stb_image (src/utils/stb_image.c, inside libsrp_ref.a), built from their
 * sources by `make -C oracle refassets`.
 *
 *   ref_assets <obj> <png> <out_dir>
 *     out_dir/teapot.bin   u64 vertexCount, u64 indexCount, then the
 *                          OBJVertex array (position, uv, normal: 8 floats)
 *                          and the u32 index array
 *     out_dir/texture.bin  i32 width, i32 height, then width*height*3 bytes,
 *                          decoded with the 3 channels srpNewTexture requests
 *                          (src/core/texture.c:26-36) */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "objparser.h"

unsigned char* stbi_load(const char* filename, int* x, int* y, int* comp, int req_comp);

int main(int argc, char** argv)
{
	if (argc != 4) { fprintf(stderr, "usage: %s <obj> <png> <out_dir>\n", argv[0]); return 2; }
	char path[4096];
	OBJMesh mesh;
	if (!loadOBJMesh(argv[1], &mesh)) { fprintf(stderr, "cannot load %s\n", argv[1]); return 1; }
	snprintf(path, sizeof path, "%s/teapot.bin", argv[3]);
	FILE* f = fopen(path, "wb");
	if (!f) return 1;
	uint64_t n[2] = { mesh.vertexCount, mesh.indexCount };
	fwrite(n, sizeof n, 1, f);
	fwrite(mesh.vertices, sizeof(OBJVertex), mesh.vertexCount, f);
	fwrite(mesh.indices, sizeof(uint32_t), mesh.indexCount, f);
	fclose(f);
	freeOBJMesh(&mesh);
	int w = 0, h = 0;
	unsigned char* rgb = stbi_load(argv[2], &w, &h, NULL, 3);
	if (!rgb) { fprintf(stderr, "cannot load %s\n", argv[2]); return 1; }
	snprintf(path, sizeof path, "%s/texture.bin", argv[3]);
	f = fopen(path, "wb");
	if (!f) return 1;
	int32_t wh[2] = { w, h };
	fwrite(wh, sizeof wh, 1, f);
	fwrite(rgb, 1, (size_t) w * h * 3, f);
	fclose(f);
	free(rgb);
	return 0;
}
