/* Tensor-core inference of the learned-shading MLP (mlp.h) for 16 pixels at
 * a time, by one warp.
 *
 * Every layer is a chain of mma.sync m16n8k16 (bf16 inputs, fp32
 * accumulation). The 16 x 64 activations of a layer never leave registers:
 * the accumulator fragment of n-tiles 2j and 2j+1 is exactly the A fragment
 * of k-chunk j of the next layer, so it is only converted to bf16 and ReLU'd
 * in place. Layer-1 A fragments are computed directly from the pixel's
 * position, normal and view direction (the sin/cos pair of one band of one
 * component sits in one register). Weights come from shared memory in the
 * transposed, padded bf16 layout of mlp.h, biases from shared memory. */
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "mlp.h"

namespace srpg {

__device__ __forceinline__ uint32_t packBf16(float lo, float hi)
{
	const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
	return *(const uint32_t*) &v;
}

__device__ __forceinline__ void mma16816(float c[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1)
{
	asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	             "{%0,%1,%2,%3};\n"
	             : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
	             : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

/* sin/cos of one band of one input component, packed as a bf16 pair (the
 * two features 2i, 2i+1 of the encoding). f is the even feature index. */
__device__ __forceinline__ uint32_t peFeaturePair(const float* x9, int f)
{
	if (f >= kMlpIn) return 0u;
	const int c = f / 12, b = (f % 12) / 2;
	float s, co;
	__sincosf(mlpBandScale(b) * x9[c], &s, &co);
	return packBf16(s, co);
}

/* in: [16][9] inputs of the slice (rows without a pixel may hold anything);
 * w: packed bf16 weights (as 32-bit pairs); bias: fp32 [64 + 64 + 64 + 3];
 * out: [16][4], RGB of each row written by the owning lanes. */
__device__ __forceinline__ void mlpSlice16(const float (*in)[9], const uint32_t* w, const float* bias, float (*out)[4])
{
	const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	const float* xg = in[g];
	const float* xh = in[g + 8];
	float acc[8][4];
	/* layer 1: K = 112 (7 k-chunks), N = 64 (8 n-tiles) */
#pragma unroll
	for (int nt = 0; nt < 8; ++nt) {
		const float b0 = bias[8 * nt + 2 * t], b1 = bias[8 * nt + 2 * t + 1];
		acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
	}
#pragma unroll
	for (int j = 0; j < kMlpInPad / 16; ++j) {
		const int f0 = 16 * j + 2 * t, f1 = f0 + 8;
		const uint32_t a0 = peFeaturePair(xg, f0), a1 = peFeaturePair(xh, f0);
		const uint32_t a2 = peFeaturePair(xg, f1), a3 = peFeaturePair(xh, f1);
#pragma unroll
		for (int nt = 0; nt < 8; ++nt) {
			const uint32_t* row = w + ((kOffT1 + (8 * nt + g) * kLd1) >> 1);
			mma16816(acc[nt], a0, a1, a2, a3, row[(16 * j + 2 * t) >> 1], row[(16 * j + 8 + 2 * t) >> 1]);
		}
	}
	/* layers 2 and 3: K = 64, N = 64, A fragments from the previous accumulators
	 * (one copy of the code for both layers) */
#pragma unroll 1
	for (int layer = 0; layer < 2; ++layer) {
		uint32_t a[4][4];
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			a[j][0] = packBf16(fmaxf(acc[2 * j][0], 0.f), fmaxf(acc[2 * j][1], 0.f));
			a[j][1] = packBf16(fmaxf(acc[2 * j][2], 0.f), fmaxf(acc[2 * j][3], 0.f));
			a[j][2] = packBf16(fmaxf(acc[2 * j + 1][0], 0.f), fmaxf(acc[2 * j + 1][1], 0.f));
			a[j][3] = packBf16(fmaxf(acc[2 * j + 1][2], 0.f), fmaxf(acc[2 * j + 1][3], 0.f));
		}
		const int wOff = layer == 0 ? kOffT2 : kOffT3;
		const float* bl = bias + kMlpHid * (1 + layer);
#pragma unroll
		for (int nt = 0; nt < 8; ++nt) {
			const float b0 = bl[8 * nt + 2 * t], b1 = bl[8 * nt + 2 * t + 1];
			acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
		}
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int nt = 0; nt < 8; ++nt) {
				const uint32_t* row = w + ((wOff + (8 * nt + g) * kLdH) >> 1);
				mma16816(acc[nt], a[j][0], a[j][1], a[j][2], a[j][3], row[(16 * j + 2 * t) >> 1],
				         row[(16 * j + 8 + 2 * t) >> 1]);
			}
	}
	/* layer 4: K = 64, N = 8 (3 used) */
	float o[4];
	{
		const float* b4 = bias + 3 * kMlpHid;
		const float b0 = 2 * t < kMlpOut ? b4[2 * t] : 0.f, b1 = 2 * t + 1 < kMlpOut ? b4[2 * t + 1] : 0.f;
		o[0] = b0; o[1] = b1; o[2] = b0; o[3] = b1;
	}
#pragma unroll
	for (int j = 0; j < 4; ++j) {
		const uint32_t a0 = packBf16(fmaxf(acc[2 * j][0], 0.f), fmaxf(acc[2 * j][1], 0.f));
		const uint32_t a1 = packBf16(fmaxf(acc[2 * j][2], 0.f), fmaxf(acc[2 * j][3], 0.f));
		const uint32_t a2 = packBf16(fmaxf(acc[2 * j + 1][0], 0.f), fmaxf(acc[2 * j + 1][1], 0.f));
		const uint32_t a3 = packBf16(fmaxf(acc[2 * j + 1][2], 0.f), fmaxf(acc[2 * j + 1][3], 0.f));
		const uint32_t* row = w + ((kOffT4 + g * kLdH) >> 1);
		mma16816(o, a0, a1, a2, a3, row[(16 * j + 2 * t) >> 1], row[(16 * j + 8 + 2 * t) >> 1]);
	}
	if (t < 2) {
		out[g][2 * t] = o[0];
		out[g + 8][2 * t] = o[2];
		if (2 * t + 1 < kMlpOut) { out[g][2 * t + 1] = o[1]; out[g + 8][2 * t + 1] = o[3]; }
	}
}

}  // namespace srpg
