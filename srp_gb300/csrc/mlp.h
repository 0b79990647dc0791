/* The learned-shading network: a small MLP that stands in for an expensive
 * fragment shader.
 *
 * Input: 6-band sin/cos positional encoding of the world position, the unit
 * normal and the unit view direction (9 components x 6 bands x 2 = 108
 * features). Three hidden layers of 64 ReLU units, 3 linear outputs (RGB,
 * clamped to [0, 1] like the shader's output).
 *
 * Parameters are kept in fp32 (training, Adam) as one flat vector:
 *   W1 [108][64], b1 [64], W2 [64][64], b2 [64], W3 [64][64], b3 [64],
 *   W4 [64][3], b4 [3]           (W[k][n]: input k, output n)
 * Inference uses a bf16 copy of the weights in the operand layout of the
 * tcgen05 tensor cores (below) and the fp32 biases. */
#pragma once

#include <stddef.h>
#include <stdint.h>

namespace srpg {

constexpr int kMlpBands = 6;
constexpr int kMlpIn = 9 * kMlpBands * 2;      /* 108 */
constexpr int kMlpInPad = 112;                /* multiple of 16 (tensor-core K step) */
constexpr int kMlpHid = 64;
constexpr int kMlpOut = 3;

/* fp32 parameter vector */
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpIn * kMlpHid;
constexpr int kOffW2 = kOffB1 + kMlpHid;
constexpr int kOffB2 = kOffW2 + kMlpHid * kMlpHid;
constexpr int kOffW3 = kOffB2 + kMlpHid;
constexpr int kOffB3 = kOffW3 + kMlpHid * kMlpHid;
constexpr int kOffW4 = kOffB3 + kMlpHid;
constexpr int kOffB4 = kOffW4 + kMlpHid * kMlpOut;
constexpr int kMlpParams = kOffB4 + kMlpOut;  /* 15491 */

/* tcgen05 operands (the canonical K-major layout of tc5.cuh), one block per
 * layer: W1 [64 n][112 k], W2 and W3 [64][64], W4 [16][64] (rows 3..15 zero);
 * one 128-row A tile; one 128 x 64 fp32 accumulator in tensor memory. */
constexpr uint32_t kTcW1 = 0;
constexpr uint32_t kTcW2 = kTcW1 + 64 * kMlpInPad * 2;
constexpr uint32_t kTcW3 = kTcW2 + 64 * 64 * 2;
constexpr uint32_t kTcW4 = kTcW3 + 64 * 64 * 2;
constexpr uint32_t kTcWBytes = kTcW4 + 16 * 64 * 2;        /* 32768 */
constexpr uint32_t kTcABytes = 128 * kMlpInPad * 2;       /* 28672 */
constexpr uint32_t kTcCols = 64;
constexpr size_t kTcSmem = kTcWBytes + kTcABytes + 208 * 4 + 16;

/* One captured fragment: world position, unit normal, unit view direction
 * and the shader's clamped RGB. */
constexpr int kSampleFloats = 12;

/* Feature f of the encoding: component c = f / 12 (position x, y, z,
 * normal x, y, z, view x, y, z), band b = (f % 12) / 2, sine for even f,
 * cosine for odd f, of 2^b * pi * value. */
#if defined(__CUDACC__)
__host__ __device__
#endif
inline float mlpBandScale(int b) { return 3.14159265358979f * (float) (1 << b); }

}  // namespace srpg
