/* Training and evaluation of the learned-shading MLP (mlp.h).
 *
 * A training step over a batch of B captured fragments:
 *   k_mlp_gather   picks B samples (hash of step and row), writes the encoded
 *                  inputs X [B][112] and the targets T [B][3]
 *   forward        H1 = relu(X W1 + b1), H2, H3 likewise, Y = H3 W4 + b4
 *   k_mlp_loss     dY = 2 (Y - T) / (3B); the squared error is summed
 *   backward       dW_l = H_{l-1}^T dH_l (split over the batch, atomics),
 *                  db_l = column sums of dH_l,
 *                  dH_{l-1} = (dH_l W_l^T) masked by H_{l-1} > 0
 *   k_mlp_adam     Adam (beta 0.9 / 0.999, eps 1e-8) with a cosine-decayed
 *                  learning rate; the step counter lives on the device
 * All matrix products go through one tiled fp32 kernel (k_mlp_gemm). Every
 * launch of a step reads its sizes and the step number from its arguments
 * or the device, so the host captures one step in a CUDA graph and replays
 * it. */
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.h"
#include "mlp_infer.cuh"

namespace srpg {

/* ------------------------------------------------------------ encoding */

__device__ __forceinline__ uint32_t mixHash(uint32_t x)
{
	x ^= x >> 16; x *= 0x7FEB352Du;
	x ^= x >> 15; x *= 0x846CA68Bu;
	x ^= x >> 16;
	return x;
}

__device__ __forceinline__ void encodeRow(const float* x9, float* row)
{
	for (int f = 0; f < kMlpIn; f += 2) {
		const int c = f / 12, b = (f % 12) / 2;
		float s, co;
		sincosf(mlpBandScale(b) * x9[c], &s, &co);
		row[f] = s;
		row[f + 1] = co;
	}
	for (int f = kMlpIn; f < kMlpInPad; ++f) row[f] = 0.0f;
}

/* One thread per batch row. Sample index: a hash of the step and the row
 * (with replacement); the step is read from the device counter. */
__global__ void k_mlp_gather(const float* samples, uint32_t nSamples, const int* step, int B, float* X, float* T)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= B) return;
	const uint32_t s = mixHash((uint32_t) *step * 0x9E3779B9u ^ mixHash((uint32_t) i + 0x632BE5ABu)) % nSamples;
	const float* in = samples + (size_t) s * kSampleFloats;
	encodeRow(in, X + (size_t) i * kMlpInPad);
	for (int k = 0; k < kMlpOut; ++k) T[(size_t) i * kMlpOut + k] = in[9 + k];
}

/* Encoded inputs of given samples, in order (evaluation). */
__global__ void k_mlp_encode(const float* samples, int n, float* X)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) encodeRow(samples + (size_t) i * kSampleFloats, X + (size_t) i * kMlpInPad);
}

/* ---------------------------------------------------------------- gemm */

enum GemmEpi { kEpiBias = 0, kEpiBiasRelu = 1, kEpiMask = 2, kEpiAtomic = 3 };

/* C[M][N] = op(A)[M][K] op(B)[K][N] with an epilogue:
 *   kEpiBias      C = acc + bias[n]
 *   kEpiBiasRelu  C = max(acc + bias[n], 0)
 *   kEpiMask      C = acc where mask[m][n] > 0, else 0
 *   kEpiAtomic    C += acc (blockIdx.z splits K into chunks of kChunk)
 * op(A) = A (A[m * lda + k]) or A^T (A[k * lda + m]); op(B) likewise. */
constexpr int kGT = 64, kGK = 16, kChunk = 512;

template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256) k_mlp_gemm(const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                                                  int M, int N, int K, const float* bias, const float* mask, int ldm)
{
	__shared__ float As[kGK][kGT + 4];
	__shared__ float Bs[kGK][kGT + 4];
	const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
	const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
	int kBeg = 0, kEnd = K;
	if (EPI == kEpiAtomic) { kBeg = blockIdx.z * kChunk; kEnd = min(K, kBeg + kChunk); }
	float acc[4][4] = {};
	for (int k0 = kBeg; k0 < kEnd; k0 += kGK) {
		for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
			const int kk = e / kGT, mm = e % kGT;
			const int k = k0 + kk, m = m0 + mm, n = n0 + mm;
			As[kk][mm] = (k < kEnd && m < M) ? (TA ? A[(size_t) k * lda + m] : A[(size_t) m * lda + k]) : 0.0f;
			Bs[kk][mm] = (k < kEnd && n < N) ? (TB ? B[(size_t) n * ldb + k] : B[(size_t) k * ldb + n]) : 0.0f;
		}
		__syncthreads();
#pragma unroll
		for (int kk = 0; kk < kGK; ++kk) {
			float a[4], b[4];
#pragma unroll
			for (int r = 0; r < 4; ++r) { a[r] = As[kk][ty * 4 + r]; b[r] = Bs[kk][tx * 4 + r]; }
#pragma unroll
			for (int r = 0; r < 4; ++r)
#pragma unroll
				for (int c = 0; c < 4; ++c) acc[r][c] += a[r] * b[c];
		}
		__syncthreads();
	}
#pragma unroll
	for (int r = 0; r < 4; ++r)
#pragma unroll
		for (int c = 0; c < 4; ++c) {
			const int m = m0 + ty * 4 + r, n = n0 + tx * 4 + c;
			if (m >= M || n >= N) continue;
			float v = acc[r][c];
			float* dst = C + (size_t) m * ldc + n;
			if (EPI == kEpiBias) *dst = v + bias[n];
			else if (EPI == kEpiBiasRelu) *dst = fmaxf(v + bias[n], 0.0f);
			else if (EPI == kEpiMask) *dst = mask[(size_t) m * ldm + n] > 0.0f ? v : 0.0f;
			else atomicAdd(dst, v);
		}
}

/* dY = 2 (Y - T) / (3B); the batch's squared error goes to *sse. */
__global__ void k_mlp_loss(const float* Y, const float* T, int B, float* dY, double* sse)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	double e = 0.0;
	if (i < B * kMlpOut) {
		const float d = Y[i] - T[i];
		dY[i] = 2.0f * d / (float) (kMlpOut * B);
		e = (double) d * d;
	}
	for (int o = 16; o; o >>= 1) e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
	if ((threadIdx.x & 31) == 0 && e != 0.0) atomicAdd(sse, e);
}

/* db[n] += sum over rows of dH[row][n] (rows split over blocks). */
__global__ void k_mlp_colsum(const float* dH, int rows, int N, float* db)
{
	const int n = threadIdx.x;
	if (n >= N) return;
	float s = 0.0f;
	for (int r = blockIdx.x; r < rows; r += gridDim.x) s += dH[(size_t) r * N + n];
	atomicAdd(&db[n], s);
}

/* Adam with a cosine-decayed rate; advances the device step counter. */
__global__ void k_mlp_adam(float* p, const float* grad, float* m, float* v, int n, int* step, int totalSteps, float lr)
{
	const int t = *step + 1;
	const float frac = totalSteps > 0 ? fminf((float) (t - 1) / (float) totalSteps, 1.0f) : 0.0f;
	const float rate = lr * 0.5f * (1.0f + cospif(frac));
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	const float c1 = 1.0f - powf(b1, (float) t), c2 = 1.0f - powf(b2, (float) t);
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float g = grad[i];
		const float mi = b1 * m[i] + (1.0f - b1) * g;
		const float vi = b2 * v[i] + (1.0f - b2) * g * g;
		m[i] = mi;
		v[i] = vi;
		p[i] -= rate * (mi / c1) / (sqrtf(vi / c2) + eps);
	}
}

__global__ void k_mlp_step_advance(int* step)
{
	if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1;
}

/* fp32 parameters -> transposed, padded bf16 weights and fp32 biases. */
__global__ void k_mlp_pack(const float* p, __nv_bfloat16* w, float* bias)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpBf16; i += gridDim.x * blockDim.x) {
		float v = 0.0f;
		if (i < kOffT2) {
			const int n = i / kLd1, k = i % kLd1;
			if (k < kMlpIn) v = p[kOffW1 + k * kMlpHid + n];
		} else if (i < kOffT4) {
			const int l = i < kOffT3 ? 0 : 1;
			const int j = i - (l ? kOffT3 : kOffT2);
			const int n = j / kLdH, k = j % kLdH;
			if (k < kMlpHid) v = p[(l ? kOffW3 : kOffW2) + k * kMlpHid + n];
		} else {
			const int j = i - kOffT4;
			const int n = j / kLdH, k = j % kLdH;
			if (n < kMlpOut && k < kMlpHid) v = p[kOffW4 + k * kMlpOut + n];
		}
		w[i] = __float2bfloat16_rn(v);
	}
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * kMlpHid + kMlpOut; i += gridDim.x * blockDim.x) {
		const int src = i < kMlpHid ? kOffB1 + i
		              : i < 2 * kMlpHid ? kOffB2 + (i - kMlpHid)
		              : i < 3 * kMlpHid ? kOffB3 + (i - 2 * kMlpHid) : kOffB4 + (i - 3 * kMlpHid);
		bias[i] = p[src];
	}
}

/* Tensor-core evaluation of n samples (tests compare it with the fp32 path):
 * one warp per 16 samples, weights staged in shared memory. */
__global__ void __launch_bounds__(128) k_mlp_eval_tc(const float* samples, int n, const __nv_bfloat16* w,
                                                     const float* bias, float* out)
{
	__shared__ uint32_t sw[kMlpBf16 / 2];
	__shared__ float sb[3 * kMlpHid + kMlpOut + 1];
	__shared__ float sin_[4][16][9];
	__shared__ float sout[4][16][4];
	for (int i = threadIdx.x; i < kMlpBf16 / 2; i += blockDim.x) sw[i] = ((const uint32_t*) w)[i];
	for (int i = threadIdx.x; i < 3 * kMlpHid + kMlpOut; i += blockDim.x) sb[i] = bias[i];
	__syncthreads();
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int base = (blockIdx.x * 4 + warp) * 16;
	if (base >= n) return;
	if (lane < 16) {
		const int r = min(base + lane, n - 1);
		for (int c = 0; c < 9; ++c) sin_[warp][lane][c] = samples[(size_t) r * kSampleFloats + c];
	}
	__syncwarp();
	mlpSlice16(sin_[warp], sw, sb, sout[warp]);
	__syncwarp();
	if (lane < 16 && base + lane < n)
		for (int c = 0; c < kMlpOut; ++c) out[(size_t) (base + lane) * kMlpOut + c] = sout[warp][lane][c];
}

}  // namespace srpg

/* ------------------------------------------------------------ launchers */

#include "mlp_ops.h"

namespace srpg {

template <bool TA, bool TB, int EPI>
static void gemm(const float* A, int lda, const float* B, int ldb, float* C, int ldc, int M, int N, int K,
                 const float* bias, const float* mask, int ldm, cudaStream_t s)
{
	const dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, EPI == kEpiAtomic ? (K + kChunk - 1) / kChunk : 1);
	k_mlp_gemm<TA, TB, EPI><<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, M, N, K, bias, mask, ldm);
}

static void colsum(const float* dH, int rows, int N, float* db, cudaStream_t s)
{
	const int blocks = rows < 256 ? (rows > 0 ? rows : 1) : 256;
	k_mlp_colsum<<<blocks, 64, 0, s>>>(dH, rows, N, db);
}

void mlpGather(const float* samples, uint32_t nSamples, const int* step, const MlpBatch& S, int B, cudaStream_t s)
{
	k_mlp_gather<<<(B + 127) / 128, 128, 0, s>>>(samples, nSamples, step, B, S.X, S.T);
}

void mlpEncode(const float* samples, int n, const MlpBatch& S, cudaStream_t s)
{
	k_mlp_encode<<<(n + 127) / 128, 128, 0, s>>>(samples, n, S.X);
}

void mlpForward(const float* p, const MlpBatch& S, int B, cudaStream_t s)
{
	gemm<false, false, kEpiBiasRelu>(S.X, kMlpInPad, p + kOffW1, kMlpHid, S.H1, kMlpHid, B, kMlpHid, kMlpIn,
	                                 p + kOffB1, nullptr, 0, s);
	gemm<false, false, kEpiBiasRelu>(S.H1, kMlpHid, p + kOffW2, kMlpHid, S.H2, kMlpHid, B, kMlpHid, kMlpHid,
	                                 p + kOffB2, nullptr, 0, s);
	gemm<false, false, kEpiBiasRelu>(S.H2, kMlpHid, p + kOffW3, kMlpHid, S.H3, kMlpHid, B, kMlpHid, kMlpHid,
	                                 p + kOffB3, nullptr, 0, s);
	gemm<false, false, kEpiBias>(S.H3, kMlpHid, p + kOffW4, kMlpOut, S.Y, kMlpOut, B, kMlpOut, kMlpHid, p + kOffB4,
	                             nullptr, 0, s);
}

void mlpBackward(const float* p, float* grad, const MlpBatch& S, int B, double* sse, cudaStream_t s)
{
	k_mlp_loss<<<(B * kMlpOut + 255) / 256, 256, 0, s>>>(S.Y, S.T, B, S.dY, sse);
	/* layer 4 */
	gemm<true, false, kEpiAtomic>(S.H3, kMlpHid, S.dY, kMlpOut, grad + kOffW4, kMlpOut, kMlpHid, kMlpOut, B, nullptr,
	                              nullptr, 0, s);
	colsum(S.dY, B, kMlpOut, grad + kOffB4, s);
	gemm<false, true, kEpiMask>(S.dY, kMlpOut, p + kOffW4, kMlpOut, S.dH3, kMlpHid, B, kMlpHid, kMlpOut, nullptr, S.H3,
	                            kMlpHid, s);
	/* layer 3 */
	gemm<true, false, kEpiAtomic>(S.H2, kMlpHid, S.dH3, kMlpHid, grad + kOffW3, kMlpHid, kMlpHid, kMlpHid, B, nullptr,
	                              nullptr, 0, s);
	colsum(S.dH3, B, kMlpHid, grad + kOffB3, s);
	gemm<false, true, kEpiMask>(S.dH3, kMlpHid, p + kOffW3, kMlpHid, S.dH2, kMlpHid, B, kMlpHid, kMlpHid, nullptr, S.H2,
	                            kMlpHid, s);
	/* layer 2 */
	gemm<true, false, kEpiAtomic>(S.H1, kMlpHid, S.dH2, kMlpHid, grad + kOffW2, kMlpHid, kMlpHid, kMlpHid, B, nullptr,
	                              nullptr, 0, s);
	colsum(S.dH2, B, kMlpHid, grad + kOffB2, s);
	gemm<false, true, kEpiMask>(S.dH2, kMlpHid, p + kOffW2, kMlpHid, S.dH1, kMlpHid, B, kMlpHid, kMlpHid, nullptr, S.H1,
	                            kMlpHid, s);
	/* layer 1 */
	gemm<true, false, kEpiAtomic>(S.X, kMlpInPad, S.dH1, kMlpHid, grad + kOffW1, kMlpHid, kMlpIn, kMlpHid, B, nullptr,
	                              nullptr, 0, s);
	colsum(S.dH1, B, kMlpHid, grad + kOffB1, s);
}

void mlpAdam(float* p, const float* grad, float* m, float* v, int* step, int totalSteps, float lr, cudaStream_t s)
{
	k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(p, grad, m, v, kMlpParams, step, totalSteps, lr);
	k_mlp_step_advance<<<1, 32, 0, s>>>(step);
}

void mlpPack(const float* p, void* w, float* bias, cudaStream_t s)
{
	k_mlp_pack<<<64, 256, 0, s>>>(p, (__nv_bfloat16*) w, bias);
}

void mlpEvalTensorCores(const float* samples, int n, const void* w, const float* bias, float* out, cudaStream_t s)
{
	if (n <= 0) return;
	k_mlp_eval_tc<<<(n + 63) / 64, 128, 0, s>>>(samples, n, (const __nv_bfloat16*) w, bias, out);
}

}  // namespace srpg
