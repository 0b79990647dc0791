/* Checks srpChainAdd (srp_gb300/csrc/chain.h) against the literal serial
 * loop it replaces, on random and adversarial (a, d, n) triples.
 * usage: chain_test <cases> <seed>; prints "ok <cases>" or the first mismatch. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "../../srp_gb300/csrc/chain.h"

static uint64_t st;
static uint64_t nx(void) { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static float rf(void)
{
	switch (nx() % 6) {
	case 0: return (float) ((double) (nx() % 2000000) / 1000000.0 - 1.0);
	case 1: { uint32_t b = (uint32_t) nx(); float f; memcpy(&f, &b, 4); return isfinite(f) ? f : 0.5f; }
	case 2: return (float) ldexp((double) (int32_t) (nx() & 0xFFFFFF) - 8388608.0, -(int) (nx() % 40));
	case 3: return (float) (nx() % 64) / 64.0f - 0.5f;
	case 4: return 0.0f;
	default: return ldexpf(1.0f, (int) (nx() % 60) - 40) * ((nx() & 1) ? 1.0f : -1.0f);
	}
}

int main(int argc, char** argv)
{
	long cases = argc > 1 ? atol(argv[1]) : 100000;
	st = argc > 2 ? strtoull(argv[2], NULL, 10) * 2654435761ull + 1 : 88172645463325252ull;
	for (long c = 0; c < cases; ++c) {
		float a = rf(), d = rf();
		if (nx() % 3 == 0) d = a * (float) ldexp(1.0, -(int) (nx() % 16)) * ((nx() & 1) ? -1.f : 1.f);
		if (nx() % 4 == 0) { float t = (float) (nx() % 4096) * 0.000244140625f; d = (nx() & 1) ? t : -t; }
		uint32_t n = (uint32_t) (nx() % 5000);
		float serial = a;
		for (uint32_t i = 0; i < n; ++i) serial = srpFAdd(serial, d);
		float fast = srpChainAdd(a, d, n);
		if (srpF2U(serial) != srpF2U(fast) && !(isnan(serial) && isnan(fast))) {
			printf("mismatch a=%a d=%a n=%u serial=%a fast=%a\n", a, d, n, serial, fast);
			return 1;
		}
	}
	printf("ok %ld\n", cases);
	return 0;
}
