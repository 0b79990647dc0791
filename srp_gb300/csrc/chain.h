/* Exact jump-ahead for a serial fp32 accumulation.
 *
 * The reference rasteriser advances barycentrics incrementally: along a row
 * lambda += dldx once per pixel, and row starts lambda_row += dldy once per
 * row (kitrofimov/srp src/raster/triangle.c:102-109). The value it tests at
 * pixel (x, y) is therefore the result of n = (x - minX) sequential
 * round-to-nearest-even additions, and the closed form l0 + n*d differs from
 * it in the last bits on most pixels. Coverage, depth and the fill rule depend
 * on those bits, so every tile of the GPU rasteriser must reproduce the chain
 * exactly, without walking it from the bounding-box corner.
 *
 * chainAdd(s, d, n) returns the value of n successive fl(s + d). It is exact:
 * while s stays inside one binade [2^e, 2^(e+1)) (same sign), every sum is
 * rounded to the same grid u = ulp(s), so each step adds the same multiple of
 * u, namely round(d / u), provided d / u is not a tie (fraction exactly 1/2)
 * and the exact sum stays strictly inside the binade. Under those conditions
 * j steps collapse into one integer add on the significand. Steps that cross
 * a binade edge, ties, zeros, subnormals and non-finite values are taken one
 * at a time with a real fp32 add. The loop costs about two iterations per
 * binade crossed, i.e. O(log(|s| / |d|)) instead of O(n).
 *
 * Host and device share this code (unit-tested against the serial loop). */
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SRP_HD __host__ __device__ __forceinline__
#else
#define SRP_HD static inline
#endif

SRP_HD uint32_t srpF2U(float f)
{
#if defined(__CUDA_ARCH__)
	return __float_as_uint(f);
#else
	uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}

SRP_HD float srpU2F(uint32_t u)
{
#if defined(__CUDA_ARCH__)
	return __uint_as_float(u);
#else
	float f; memcpy(&f, &u, 4); return f;
#endif
}

/* One round-to-nearest fp32 add, never contracted. */
SRP_HD float srpFAdd(float a, float b)
{
#if defined(__CUDA_ARCH__)
	return __fadd_rn(a, b);
#else
	volatile float r = a + b;
	return r;
#endif
}

/* Number of serial steps below which the plain loop is used. */
#define SRP_CHAIN_SERIAL 32

SRP_HD float srpChainAdd(float s, float d, uint32_t n)
{
	while (n > 0) {
		if (n <= SRP_CHAIN_SERIAL) {
			for (uint32_t i = 0; i < n; ++i) s = srpFAdd(s, d);
			return s;
		}
		const float t = srpFAdd(s, d);
		const uint32_t bs = srpF2U(s), bt = srpF2U(t);
		if (bs == bt) return s;  /* fixed point: all further adds leave s unchanged */
		const uint32_t es = (bs >> 23) & 0xFFu, et = (bt >> 23) & 0xFFu;
		if (((bs ^ bt) >> 31) == 0 && es == et && es != 0 && es != 0xFFu) {
			/* tie test: does d fall exactly half-way between multiples of u? */
			const uint32_t bd = srpF2U(d);
			uint32_t ed = (bd >> 23) & 0xFFu;
			const uint32_t md = (bd & 0x7FFFFFu) | (ed ? 0x800000u : 0u);
			if (ed == 0) ed = 1;
			int tie = 0;
			if (ed < es) {
				const uint32_t k = es - ed;
				if (k <= 25u) tie = (md & ((1u << k) - 1u)) == (1u << (k - 1u));
			}
			if (!tie) {
				/* significands in units of u; the walk must stay in [2^23 + 1, 2^24 - 1] */
				const int32_t S = (int32_t) ((bs & 0x7FFFFFu) | 0x800000u);
				const int32_t T = (int32_t) ((bt & 0x7FFFFFu) | 0x800000u);
				const int32_t D = T - S;
				const int32_t m = D > 0 ? (0xFFFFFF - S) / D : (S - 0x800001) / (-D);
				if (m >= 1) {
					const uint32_t j = (uint32_t) m < n ? (uint32_t) m : n;
					const int32_t Sj = S + (int32_t) j * D;
					s = srpU2F((bs & 0xFF800000u) | ((uint32_t) Sj & 0x7FFFFFu));
					n -= j;
					continue;
				}
			}
		}
		s = t;
		n -= 1;
	}
	return s;
}
