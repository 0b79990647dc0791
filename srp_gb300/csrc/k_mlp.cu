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
#include "tc5.cuh"

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

/* fp32 biases of the four layers, in one array [64 + 64 + 64 + 3]. */
__global__ void k_mlp_pack_bias(const float* p, float* bias)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * kMlpHid + kMlpOut; i += gridDim.x * blockDim.x) {
		const int src = i < kMlpHid ? kOffB1 + i
		              : i < 2 * kMlpHid ? kOffB2 + (i - kMlpHid)
		              : i < 3 * kMlpHid ? kOffB3 + (i - 2 * kMlpHid) : kOffB4 + (i - 3 * kMlpHid);
		bias[i] = p[src];
	}
}

/* ------------------------------------------------- tcgen05 evaluation */


__global__ void k_mlp_pack5(const float* p, uint8_t* out)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (int) (kTcWBytes / 2); i += gridDim.x * blockDim.x) {
		/* which layer, and (n, k) inside it, for bf16 slot i */
		const uint32_t byte = 2u * (uint32_t) i;
		uint32_t base, K;
		int layer;
		if (byte < kTcW2) { base = kTcW1; K = kMlpInPad; layer = 0; }
		else if (byte < kTcW3) { base = kTcW2; K = 64; layer = 1; }
		else if (byte < kTcW4) { base = kTcW3; K = 64; layer = 2; }
		else { base = kTcW4; K = 64; layer = 3; }
		const uint32_t off = byte - base;
		const uint32_t sbo = K / 8 * 128;
		const int rg = (int) (off / sbo), rem = (int) (off % sbo);
		const int kc = rem / 128, rr = (rem % 128) / 16, kk = (rem % 16) / 2;
		const int n = rg * 8 + rr, k = kc * 8 + kk;
		float v = 0.0f;
		if (layer == 0) { if (k < kMlpIn) v = p[kOffW1 + k * kMlpHid + n]; }
		else if (layer == 1) v = p[kOffW2 + k * kMlpHid + n];
		else if (layer == 2) v = p[kOffW3 + k * kMlpHid + n];
		else if (n < kMlpOut) v = p[kOffW4 + k * kMlpOut + n];
		((__nv_bfloat16*) out)[i] = __float2bfloat16_rn(v);
	}
}

/* Evaluation of n samples, 128 per step, on tcgen05: the encoded inputs of a
 * step form one 128-row A tile, every layer is one chain of K/16 MMAs into a
 * 128 x 64 fp32 accumulator in tensor memory, and each warp moves its 32
 * rows back through registers (bias, ReLU, bf16) into the next A tile. */
__global__ void __launch_bounds__(128) k_mlp_eval_tc5(const float* samples, int n, const uint8_t* w5, const float* bias,
                                                      float* out, unsigned* err)
{
	extern __shared__ __align__(1024) uint8_t tsm[];
	uint8_t* sW = tsm;
	uint8_t* sA = tsm + kTcWBytes;
	float* sB = (float*) (sA + kTcABytes);
	uint64_t* mbar = (uint64_t*) (sB + 208);
	uint32_t* tslot = (uint32_t*) (mbar + 1);
	const int tid = threadIdx.x, warp = tid >> 5;
	for (int i = tid; i < (int) (kTcWBytes / 16); i += 128) ((uint4*) sW)[i] = ((const uint4*) w5)[i];
	for (int i = tid; i < 3 * kMlpHid + kMlpOut; i += 128) sB[i] = bias[i];
	const uint32_t mb = smemAddr(mbar);
	if (tid == 0) mbarInit(mb, 1);
	if (warp == 0) tcAlloc(smemAddr(tslot), kTcCols);
	fenceProxyAsync();
	tcFenceBefore();
	__syncthreads();
	tcFenceAfter();
	const uint32_t tmem = *tslot;
	const uint32_t laneBase = tmem + ((uint32_t) (warp * 32) << 16);
	const uint32_t aAddr = smemAddr(sA), wAddr = smemAddr(sW);
	uint32_t phase = 0;
	bool ok = true;
	for (int tile = blockIdx.x; tile * 128 < n; tile += gridDim.x) {
		const int r = tid, s = tile * 128 + r;
		const float* x9 = samples + (size_t) min(s, n - 1) * kSampleFloats;
		for (int f = 0; f < kMlpInPad; f += 2) {
			uint32_t v = 0;
			if (f < kMlpIn) {
				float sn, cs;
				__sincosf(mlpBandScale((f % 12) / 2) * x9[f / 12], &sn, &cs);
				v = packBf16(sn, cs);
			}
			*(uint32_t*) (sA + tcOffset(r, f, kMlpInPad)) = v;
		}
		fenceProxyAsync();
		tcFenceBefore();
		__syncthreads();
		for (int layer = 0; layer < 4; ++layer) {
			if (tid == 0) {
				tcFenceAfter();
				const int K = layer == 0 ? kMlpInPad : 64;
				const uint32_t w = wAddr + (layer == 0 ? kTcW1 : layer == 1 ? kTcW2 : layer == 2 ? kTcW3 : kTcW4);
				tcLayer(tmem, aAddr, w, K, layer < 3 ? 64 : 16);
				tcCommit(mb);
			}
			const bool got = mbarWait(mb, phase);
			phase ^= 1u;
			if (!__syncthreads_and(got)) { ok = false; break; }
			tcFenceAfter();
			if (layer < 3) {
				/* this thread's row: bias, ReLU, bf16 into the next A tile */
				const float* b = sB + 64 * layer;
				for (int c = 0; c < 64; c += 16) {
					float v[16];
					tcLoad16(laneBase + (uint32_t) c, v);
#pragma unroll
					for (int i = 0; i < 16; i += 2) {
						const float x0 = fmaxf(v[i] + b[c + i], 0.0f), x1 = fmaxf(v[i + 1] + b[c + i + 1], 0.0f);
						*(uint32_t*) (sA + tcOffset(r, c + i, 64)) = packBf16(x0, x1);
					}
				}
				fenceProxyAsync();
				tcFenceBefore();
				__syncthreads();
			} else {
				float v[16];
				tcLoad16(laneBase, v);
				if (s < n)
					for (int k = 0; k < kMlpOut; ++k) out[(size_t) s * kMlpOut + k] = v[k] + sB[3 * kMlpHid + k];
				tcFenceBefore();
				__syncthreads();
			}
		}
		if (!ok) break;
	}
	if (!ok && tid == 0) atomicOr(err, 1u);
	tcFenceBefore();
	__syncthreads();
	tcFenceAfter();
	if (warp == 0) tcDealloc(tmem, kTcCols);
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

void mlpPack5(const float* params, void* w5, float* bias, cudaStream_t s)
{
	k_mlp_pack5<<<64, 256, 0, s>>>(params, (uint8_t*) w5);
	k_mlp_pack_bias<<<1, 256, 0, s>>>(params, bias);
}

void mlpEvalTcgen05(const float* samples, int n, const void* w5, const float* bias, float* out, unsigned* err,
                    cudaStream_t s)
{
	if (n <= 0) return;
	cudaFuncSetAttribute(k_mlp_eval_tc5, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kTcSmem);
	const int tiles = (n + 127) / 128;
	k_mlp_eval_tc5<<<tiles < 152 * 3 ? tiles : 152 * 3, 128, kTcSmem, s>>>(samples, n, (const uint8_t*) w5, bias, out,
	                                                                        err);
}

}  // namespace srpg
