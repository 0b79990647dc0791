/* Minimal image decoding for srpNewTexture: binary PPM (P6, maxval 255) and,
 * when zlib is available (SRP_HAVE_ZLIB), 8-bit non-interlaced PNG (grey,
 * grey+alpha, RGB, RGBA, palette). Output is always 3 channels (RGB8),
 * row-major, top row first, which is what the reference's texture loader
 * requests (kitrofimov/srp src/core/texture.c:25,34). Decoding an image is not
 * part of the draw path; it only has to deliver the same texel bytes. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "imageio.h"
#ifdef SRP_HAVE_ZLIB
#include <zlib.h>
#endif

static unsigned char* read_file(const char* path, size_t* n)
{
	FILE* f = fopen(path, "rb");
	if (!f) return NULL;
	fseek(f, 0, SEEK_END);
	long len = ftell(f);
	fseek(f, 0, SEEK_SET);
	if (len <= 0) { fclose(f); return NULL; }
	unsigned char* buf = (unsigned char*) malloc((size_t) len);
	if (buf && fread(buf, 1, (size_t) len, f) != (size_t) len) { free(buf); buf = NULL; }
	fclose(f);
	*n = (size_t) len;
	return buf;
}

static const unsigned char* ppm_token(const unsigned char* p, const unsigned char* end, long* out)
{
	for (;;) {
		while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
		if (p < end && *p == '#') { while (p < end && *p != '\n') ++p; continue; }
		break;
	}
	if (p >= end || *p < '0' || *p > '9') return NULL;
	long v = 0;
	while (p < end && *p >= '0' && *p <= '9') v = v * 10 + (*p++ - '0');
	*out = v;
	return p;
}

static int decode_ppm(const unsigned char* d, size_t n, SRPImage* img, const char** err)
{
	const unsigned char* p = d + 2;
	const unsigned char* end = d + n;
	long w, h, maxv;
	if (!(p = ppm_token(p, end, &w)) || !(p = ppm_token(p, end, &h)) || !(p = ppm_token(p, end, &maxv)))
		{ *err = "malformed PPM header"; return 0; }
	if (maxv != 255 || w <= 0 || h <= 0) { *err = "unsupported PPM (maxval must be 255)"; return 0; }
	++p; /* single whitespace after maxval */
	size_t bytes = (size_t) w * (size_t) h * 3;
	if ((size_t) (end - p) < bytes) { *err = "truncated PPM"; return 0; }
	img->rgb = (uint8_t*) malloc(bytes);
	memcpy(img->rgb, p, bytes);
	img->width = (int) w;
	img->height = (int) h;
	return 1;
}

#ifdef SRP_HAVE_ZLIB
static uint32_t be32(const unsigned char* p) { return (uint32_t) p[0] << 24 | (uint32_t) p[1] << 16 | (uint32_t) p[2] << 8 | p[3]; }

static int paeth(int a, int b, int c)
{
	int p = a + b - c, pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
	if (pa <= pb && pa <= pc) return a;
	return pb <= pc ? b : c;
}

static int decode_png(const unsigned char* d, size_t n, SRPImage* img, const char** err)
{
	size_t pos = 8;
	uint32_t w = 0, h = 0;
	int depth = 0, ctype = -1, interlace = 0;
	unsigned char plte[768];
	int nplte = 0;
	unsigned char* idat = NULL;
	size_t nidat = 0;
	while (pos + 12 <= n) {
		uint32_t len = be32(d + pos);
		const unsigned char* type = d + pos + 4;
		const unsigned char* body = d + pos + 8;
		if (pos + 12 + (size_t) len > n) break;
		if (!memcmp(type, "IHDR", 4) && len >= 13) {
			w = be32(body); h = be32(body + 4);
			depth = body[8]; ctype = body[9]; interlace = body[12];
		} else if (!memcmp(type, "PLTE", 4) && len <= 768) {
			memcpy(plte, body, len); nplte = (int) (len / 3);
		} else if (!memcmp(type, "IDAT", 4)) {
			idat = (unsigned char*) realloc(idat, nidat + len);
			memcpy(idat + nidat, body, len);
			nidat += len;
		} else if (!memcmp(type, "IEND", 4)) break;
		pos += 12 + (size_t) len;
	}
	int ch = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
	if (!w || !h || depth != 8 || !ch || interlace || !idat)
		{ free(idat); *err = "unsupported PNG (needs 8-bit, non-interlaced)"; return 0; }
	size_t stride = (size_t) w * (size_t) ch;
	uLongf rawlen = (uLongf) ((stride + 1) * h);
	unsigned char* raw = (unsigned char*) malloc(rawlen);
	if (uncompress(raw, &rawlen, idat, (uLong) nidat) != Z_OK || rawlen != (stride + 1) * h)
		{ free(idat); free(raw); *err = "corrupt PNG data"; return 0; }
	free(idat);
	unsigned char* pix = (unsigned char*) malloc(stride * h);
	for (uint32_t y = 0; y < h; ++y) {
		unsigned char f = raw[y * (stride + 1)];
		const unsigned char* src = raw + y * (stride + 1) + 1;
		unsigned char* row = pix + y * stride;
		const unsigned char* up = y ? pix + (y - 1) * stride : NULL;
		for (size_t i = 0; i < stride; ++i) {
			int a = i >= (size_t) ch ? row[i - ch] : 0;
			int b = up ? up[i] : 0;
			int c = (up && i >= (size_t) ch) ? up[i - ch] : 0;
			int v = src[i];
			switch (f) {
			case 1: v += a; break;
			case 2: v += b; break;
			case 3: v += (a + b) >> 1; break;
			case 4: v += paeth(a, b, c); break;
			default: break;
			}
			row[i] = (unsigned char) v;
		}
	}
	free(raw);
	img->rgb = (uint8_t*) malloc((size_t) w * h * 3);
	for (size_t i = 0; i < (size_t) w * h; ++i) {
		const unsigned char* s = pix + i * ch;
		uint8_t* o = img->rgb + i * 3;
		if (ctype == 3) {
			int k = s[0] < nplte ? s[0] : 0;
			o[0] = plte[3 * k]; o[1] = plte[3 * k + 1]; o[2] = plte[3 * k + 2];
		} else if (ch <= 2) {
			o[0] = o[1] = o[2] = s[0];
		} else {
			o[0] = s[0]; o[1] = s[1]; o[2] = s[2];
		}
	}
	free(pix);
	img->width = (int) w;
	img->height = (int) h;
	return 1;
}
#endif

int srpImageLoad(const char* path, SRPImage* img, const char** err)
{
	size_t n = 0;
	unsigned char* d = read_file(path, &n);
	img->rgb = NULL;
	if (!d) { *err = "cannot read file"; return 0; }
	int ok = 0;
	if (n >= 2 && d[0] == 'P' && d[1] == '6')
		ok = decode_ppm(d, n, img, err);
#ifdef SRP_HAVE_ZLIB
	else if (n >= 8 && !memcmp(d, "\x89PNG\r\n\x1a\n", 8))
		ok = decode_png(d, n, img, err);
#endif
	else
		*err = "unsupported image format (PPM P6, or PNG when built with zlib)";
	free(d);
	return ok;
}

int srpImageWritePPM(const char* path, const uint8_t* rgb, int width, int height)
{
	FILE* f = fopen(path, "wb");
	if (!f) return 0;
	fprintf(f, "P6\n%d %d\n255\n", width, height);
	size_t bytes = (size_t) width * height * 3;
	int ok = fwrite(rgb, 1, bytes, f) == bytes;
	fclose(f);
	return ok;
}

/* ------------------------------------------------------------ PNG writer */

/* CRC-32 (ISO 3309, as PNG chunks use it), bitwise. */
static uint32_t png_crc(uint32_t crc, const unsigned char* p, size_t n)
{
	crc = ~crc;
	for (size_t i = 0; i < n; ++i) {
		crc ^= p[i];
		for (int k = 0; k < 8; ++k) crc = (crc >> 1) ^ (0xEDB88320u & (0u - (crc & 1u)));
	}
	return ~crc;
}

static void put32(unsigned char* p, uint32_t v)
{
	p[0] = (unsigned char) (v >> 24); p[1] = (unsigned char) (v >> 16);
	p[2] = (unsigned char) (v >> 8); p[3] = (unsigned char) v;
}

static int png_chunk(FILE* f, const char* type, const unsigned char* data, size_t n)
{
	unsigned char hdr[8];
	put32(hdr, (uint32_t) n);
	memcpy(hdr + 4, type, 4);
	uint32_t crc = png_crc(0, hdr + 4, 4);
	crc = png_crc(crc, data, n);
	unsigned char tail[4];
	put32(tail, crc);
	return fwrite(hdr, 1, 8, f) == 8 && (n == 0 || fwrite(data, 1, n, f) == n) && fwrite(tail, 1, 4, f) == 4;
}

int srpImageWritePNG(const char* path, const uint8_t* rgba, int width, int height)
{
	if (width <= 0 || height <= 0) return 0;
	/* filter byte 0 (none) before every row of RGBA8 */
	const size_t row = (size_t) width * 4 + 1, raw = row * (size_t) height;
	/* zlib stream of stored deflate blocks (at most 65535 bytes each) */
	const size_t blocks = (raw + 65534) / 65535;
	const size_t zn = 2 + raw + blocks * 5 + 4;
	unsigned char* z = (unsigned char*) malloc(zn);
	if (!z) return 0;
	size_t o = 0;
	z[o++] = 0x78; z[o++] = 0x01;
	uint32_t a = 1, b = 0;   /* Adler-32 of the uncompressed bytes */
	size_t done = 0;
	for (int y = 0; y < height; ++y) {
		for (size_t i = 0; i < row; ++i) {
			if (done % 65535 == 0) {
				const size_t len = raw - done < 65535 ? raw - done : 65535;
				z[o++] = (unsigned char) (done + len == raw ? 1 : 0);
				z[o++] = (unsigned char) len; z[o++] = (unsigned char) (len >> 8);
				z[o++] = (unsigned char) ~len; z[o++] = (unsigned char) (~len >> 8);
			}
			const unsigned char v = i == 0 ? 0 : rgba[(size_t) y * width * 4 + (i - 1)];
			z[o++] = v;
			a = (a + v) % 65521u;
			b = (b + a) % 65521u;
			++done;
		}
	}
	put32(z + o, (b << 16) | a);
	o += 4;
	FILE* f = fopen(path, "wb");
	if (!f) { free(z); return 0; }
	unsigned char ihdr[13];
	put32(ihdr, (uint32_t) width);
	put32(ihdr + 4, (uint32_t) height);
	ihdr[8] = 8; ihdr[9] = 6; ihdr[10] = 0; ihdr[11] = 0; ihdr[12] = 0;   /* RGBA8, no interlace */
	int ok = fwrite("\x89PNG\r\n\x1a\n", 1, 8, f) == 8 && png_chunk(f, "IHDR", ihdr, 13) &&
	         png_chunk(f, "IDAT", z, o) && png_chunk(f, "IEND", NULL, 0);
	ok = fclose(f) == 0 && ok;
	free(z);
	return ok;
}
