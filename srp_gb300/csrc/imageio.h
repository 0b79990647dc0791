/* Image decoding used by srpNewTexture (not part of the draw path). */
#pragma once
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct SRPImage { uint8_t* rgb; int width; int height; } SRPImage;
/* Decode `path` into 3-channel RGB8. Returns 1 on success, else 0 and *err. */
int srpImageLoad(const char* path, SRPImage* img, const char** err);
/* Write RGB8 as binary PPM. Returns 1 on success. */
int srpImageWritePPM(const char* path, const uint8_t* rgb, int width, int height);
/* Write RGBA8 rows (top first) as a PNG of stored (uncompressed) deflate
 * blocks; needs no zlib. Returns 1 on success. */
int srpImageWritePNG(const char* path, const uint8_t* rgba, int width, int height);
#ifdef __cplusplus
}
#endif
