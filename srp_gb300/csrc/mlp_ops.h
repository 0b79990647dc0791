/* Host-side launchers of the learned-shading network's kernels (k_mlp.cu). */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.h"

namespace srpg {

/* Device scratch of one batch of B rows: encoded inputs, targets, layer
 * outputs and their gradients. */
struct MlpBatch {
	float* X;     /* [B][kMlpInPad] */
	float* T;     /* [B][3] */
	float* H1;    /* [B][64] each */
	float* H2;
	float* H3;
	float* Y;     /* [B][3] */
	float* dY;
	float* dH3;
	float* dH2;
	float* dH1;
};

void mlpGather(const float* samples, uint32_t nSamples, const int* step, const MlpBatch& S, int B, cudaStream_t s);
void mlpEncode(const float* samples, int n, const MlpBatch& S, cudaStream_t s);
void mlpForward(const float* params, const MlpBatch& S, int B, cudaStream_t s);
/* gradients accumulate into grad (zero it first); the batch's squared error
 * is added to *sse */
void mlpBackward(const float* params, float* grad, const MlpBatch& S, int B, double* sse, cudaStream_t s);
void mlpAdam(float* params, const float* grad, float* m, float* v, int* step, int totalSteps, float lr, cudaStream_t s);
/* bf16 weights in the tcgen05 operand layout of tc5.cuh (32768 bytes) and
 * fp32 biases [64 + 64 + 64 + 3] */
void mlpPack5(const float* params, void* w5, float* bias, cudaStream_t s);
void mlpEvalTcgen05(const float* samples, int n, const void* w5, const float* bias, float* out, unsigned* err,
                    cudaStream_t s);

}  // namespace srpg
