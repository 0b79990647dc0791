/* Learned shading: a small MLP (mlp.h) trained on the GPU on fragments that
 * an expensive fragment shader produced, then used in its place.
 *
 *   capture   while enabled, draws shaded by the target shader record 1 of
 *             every N shaded pixels (position, normal, view direction,
 *             colour) into the network's sample buffer (k_shade, k_raster.cu)
 *   train     Adam over random batches of the samples (k_mlp.cu); one step is
 *             captured in a CUDA graph and replayed
 *   shade     draws whose fragment shader is the target are shaded by the
 *             network on the tcgen05 tensor cores (k_shade_learned5); 1 pixel in
 *             judgeEvery is shaded by the target as well, and a draw whose
 *             PSNR over those pixels is below the threshold is shaded again
 *             by the target alone (fallback)
 * Coverage, depth, stencil and the choice of the visible fragment never
 * depend on the network: only the colour of the visible fragment does.
 *
 * Nothing here has a counterpart in kitrofimov/srp. */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "srp/gpu.h"
#include "kernels.h"
#include "learned_internal.h"
#include "mlp.h"
#include "mlp_ops.h"

using namespace srpg;

struct SRPGpuMlp {
	float* params = nullptr;     /* fp32 master copy [kMlpParams] */
	float* adamM = nullptr;
	float* adamV = nullptr;
	float* grad = nullptr;
	void* packed5 = nullptr;     /* bf16 weights in the tcgen05 operand layout (32768 bytes) */
	unsigned* tcErr = nullptr;   /* set by a tcgen05 kernel whose wait gave up */
	float* bias = nullptr;       /* fp32 biases [3 * 64 + 3 + 1] */
	float* samples = nullptr;    /* [capacity][kSampleFloats] */
	unsigned long long* count = nullptr;
	size_t capacity = 0;
	int* step = nullptr;
	double* sse = nullptr;
	MlpBatch batch = {};
	int batchCap = 0;
	cudaStream_t stream = nullptr;
	cudaGraphExec_t graph = nullptr;
	int graphBatch = 0, graphSteps = 0;
	size_t graphSamples = 0;
	float graphLr = 0.0f;
	bool packedValid = false;
};

namespace {

struct Learned {
	/* capture */
	SRPGpuMlp* capture = nullptr;
	int captureFs = 0;
	uint32_t captureEvery = 64;
	/* shading */
	SRPGpuMlp* net = nullptr;
	int targetFs = 0;
	float minPsnr = 40.0f;
	uint32_t judgeEvery = 64;
	double* judge = nullptr;          /* [2 * judgeCap] */
	unsigned int* judgeMax = nullptr; /* [judgeCap] */
	uint32_t judgeCap = 0;
	uint8_t* redoDev = nullptr;
	std::vector<double> hostJudge;
	std::vector<unsigned int> hostMax;
	SRPGpuLearnedStats stats = {};
};

Learned L;

bool ok(cudaError_t e, const char* what)
{
	if (e == cudaSuccess) return true;
	learnedError("%s: %s", what, cudaGetErrorString(e));
	return false;
}

template <class T> bool devAlloc(T** p, size_t n, const char* what)
{
	return ok(cudaMalloc((void**) p, n * sizeof(T) + 16), what);
}

bool reserveBatch(SRPGpuMlp* m, int B)
{
	if (B <= m->batchCap) return true;
	MlpBatch& S = m->batch;
	float** bufs[] = { &S.X, &S.T, &S.H1, &S.H2, &S.H3, &S.Y, &S.dY, &S.dH3, &S.dH2, &S.dH1 };
	const size_t cols[] = { (size_t) kMlpInPad, kMlpOut, kMlpHid, kMlpHid, kMlpHid, kMlpOut, kMlpOut, kMlpHid, kMlpHid,
	                        kMlpHid };
	for (int i = 0; i < 10; ++i) {
		if (*bufs[i]) cudaFree(*bufs[i]);
		*bufs[i] = nullptr;
		if (!devAlloc(bufs[i], (size_t) B * cols[i], "srpGpuMlp batch")) return false;
	}
	m->batchCap = B;
	if (m->graph) { cudaGraphExecDestroy(m->graph); m->graph = nullptr; }
	return true;
}

bool ensureJudge(uint32_t n)
{
	if (n <= L.judgeCap) return true;
	if (L.judge) cudaFree(L.judge);
	if (L.judgeMax) cudaFree(L.judgeMax);
	if (L.redoDev) cudaFree(L.redoDev);
	L.judge = nullptr; L.judgeMax = nullptr; L.redoDev = nullptr;
	const uint32_t cap = n < 64 ? 64 : n;
	if (!devAlloc(&L.judge, 2 * (size_t) cap, "judge") || !devAlloc(&L.judgeMax, cap, "judge") ||
	    !devAlloc(&L.redoDev, cap, "judge"))
		return false;
	L.judgeCap = cap;
	return true;
}

bool packIfNeeded(SRPGpuMlp* m)
{
	if (m->packedValid) return true;
	mlpPack5(m->params, m->packed5, m->bias, m->stream);
	if (!ok(cudaStreamSynchronize(m->stream), "srpGpuMlp pack")) return false;
	m->packedValid = true;
	return true;
}

}  // namespace

/* ----------------------------------------------------- hooks of the draw */

namespace srpg {

bool learnedPrepare(DrawParams& P, int kind, bool late, uint32_t nDraws, cudaStream_t s)
{
	P.capture = nullptr;
	P.mlpW5 = nullptr;
	P.redo = nullptr;
	/* the pixels sampled for capture and judging follow a fixed hash of the
	 * pixel and the draw, so a repeated draw has the same parameters */
	P.sampleSeed = 0x51ED270Bu;
	if (L.capture && P.fsId == L.captureFs && kind == kKindTri) {
		P.capture = L.capture->samples;
		P.captureCount = L.capture->count;
		P.captureCap = (uint32_t) (L.capture->capacity < 0xFFFFFFFFull ? L.capture->capacity : 0xFFFFFFFFull);
		P.captureEvery = L.captureEvery;
	}
	if (!L.net || P.fsId != L.targetFs || kind != kKindTri || late) return false;
	if (!ensureJudge(nDraws) || !packIfNeeded(L.net)) return false;
	cudaMemsetAsync(L.judge, 0, 2 * sizeof(double) * nDraws, s);
	cudaMemsetAsync(L.judgeMax, 0, sizeof(unsigned int) * nDraws, s);
	P.judgeFs = P.fsId;
	P.fsId = kFsLearned;
	P.mlpW5 = L.net->packed5;
	P.mlpB = L.net->bias;
	P.judge = L.judge;
	P.judgeMax = L.judgeMax;
	P.judgeEvery = L.judgeEvery;
	return true;
}

uint32_t learnedJudge(uint32_t nDraws, uint8_t* redo, const uint8_t** redoDev, cudaStream_t s,
                      const DeviceCounters* ctr)
{
	L.hostJudge.resize(2 * (size_t) nDraws);
	L.hostMax.resize(nDraws);
	unsigned int errors = 0;
	cudaMemcpyAsync(L.hostJudge.data(), L.judge, 2 * sizeof(double) * nDraws, cudaMemcpyDeviceToHost, s);
	cudaMemcpyAsync(L.hostMax.data(), L.judgeMax, sizeof(unsigned int) * nDraws, cudaMemcpyDeviceToHost, s);
	cudaMemcpyAsync(&errors, &ctr->errors, sizeof errors, cudaMemcpyDeviceToHost, s);
	if (!ok(cudaStreamSynchronize(s), "learned shading judge")) return 0;
	if (errors & kErrSpin) {
		/* the network's colours are incomplete: every draw is shaded again */
		learnedError("a tensor-core wait of the learned shading kernel timed out; the draw%s shaded again by "
		             "its own fragment shader", nDraws > 1 ? "s are" : " is");
		for (uint32_t d = 0; d < nDraws; ++d) redo[d] = 1;
		L.stats.draws += nDraws;
		L.stats.fallbacks += nDraws;
		if (redoDev) {
			cudaMemcpyAsync(L.redoDev, redo, nDraws, cudaMemcpyHostToDevice, s);
			*redoDev = L.redoDev;
		}
		return nDraws;
	}
	uint32_t nRedo = 0;
	for (uint32_t d = 0; d < nDraws; ++d) {
		const double sse = L.hostJudge[2 * d], chans = L.hostJudge[2 * d + 1];
		float worst;
		memcpy(&worst, &L.hostMax[d], 4);
		/* PSNR over [0, 1] channels; no judged pixel means nothing to judge */
		const double mse = chans > 0 ? sse / chans : 0.0;
		const double psnr = mse > 0 ? 10.0 * log10(1.0 / mse) : 200.0;
		const bool bad = chans > 0 && psnr < (double) L.minPsnr;
		redo[d] = bad ? 1 : 0;
		nRedo += bad;
		SRPGpuLearnedStats& st = L.stats;
		if (chans > 0) {
			st.judgedChannels += (uint64_t) chans;
			st.squaredError += sse;
			st.lastPsnrDb = psnr;
			if (st.judgedDraws == 0 || psnr < st.minPsnrDb) st.minPsnrDb = psnr;
			++st.judgedDraws;
			const int bin = psnr < 20 ? 0 : psnr < 25 ? 1 : psnr < 30 ? 2 : psnr < 35 ? 3 : psnr < 40 ? 4 : 5;
			++st.psnrHistogram[bin];
		}
		if (worst > st.maxChannelError) st.maxChannelError = worst;
		++st.draws;
		st.fallbacks += bad;
	}
	if (nRedo && redoDev) {
		cudaMemcpyAsync(L.redoDev, redo, nDraws, cudaMemcpyHostToDevice, s);
		*redoDev = L.redoDev;
	}
	return nRedo;
}

}  // namespace srpg

/* ------------------------------------------------------------- C API */

extern "C" {

SRPGpuMlp* srpGpuMlpCreate(uint64_t seed, size_t sampleCapacity)
{
	SRPGpuMlp* m = new SRPGpuMlp();
	bool good = ok(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "srpGpuMlpCreate") &&
	            devAlloc(&m->params, kMlpParams, "srpGpuMlpCreate") && devAlloc(&m->adamM, kMlpParams, "srpGpuMlpCreate") &&
	            devAlloc(&m->adamV, kMlpParams, "srpGpuMlpCreate") && devAlloc(&m->grad, kMlpParams, "srpGpuMlpCreate") &&
	            ok(cudaMalloc(&m->packed5, 32768 + 16), "srpGpuMlpCreate") && devAlloc(&m->tcErr, 1, "srpGpuMlpCreate") &&
	            devAlloc(&m->bias, 3 * kMlpHid + kMlpOut + 1, "srpGpuMlpCreate") &&
	            devAlloc(&m->count, 1, "srpGpuMlpCreate") && devAlloc(&m->step, 1, "srpGpuMlpCreate") &&
	            devAlloc(&m->sse, 1, "srpGpuMlpCreate") &&
	            devAlloc(&m->samples, (sampleCapacity ? sampleCapacity : 1) * kSampleFloats, "srpGpuMlpCreate");
	if (!good) { srpGpuMlpFree(m); return nullptr; }
	m->capacity = sampleCapacity;
	/* uniform init scaled by fan-in (He), biases zero; splitmix64 draws */
	std::vector<float> p(kMlpParams, 0.0f);
	uint64_t x = seed * 0x9E3779B97F4A7C15ull + 0xD1B54A32D192ED03ull;
	auto next = [&x]() {
		uint64_t z = (x += 0x9E3779B97F4A7C15ull);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		return z ^ (z >> 31);
	};
	auto fill = [&](int off, int fanIn, int n) {
		const double a = sqrt(6.0 / fanIn);
		for (int i = 0; i < n; ++i) p[off + i] = (float) (((double) (next() >> 11) / 9007199254740992.0 * 2.0 - 1.0) * a);
	};
	fill(kOffW1, kMlpIn, kMlpIn * kMlpHid);
	fill(kOffW2, kMlpHid, kMlpHid * kMlpHid);
	fill(kOffW3, kMlpHid, kMlpHid * kMlpHid);
	fill(kOffW4, kMlpHid, kMlpHid * kMlpOut);
	cudaMemcpy(m->params, p.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
	cudaMemset(m->count, 0, sizeof(unsigned long long));
	return m;
}

void srpGpuMlpFree(SRPGpuMlp* m)
{
	if (!m) return;
	if (L.capture == m) L.capture = nullptr;
	if (L.net == m) L.net = nullptr;
	if (m->stream) cudaStreamSynchronize(m->stream);
	if (m->graph) cudaGraphExecDestroy(m->graph);
	void* bufs[] = { m->params, m->adamM, m->adamV, m->grad, m->packed5, m->tcErr, m->bias, m->samples,
	                 m->count, m->step, m->sse,
	                 m->batch.X, m->batch.T, m->batch.H1, m->batch.H2, m->batch.H3, m->batch.Y, m->batch.dY,
	                 m->batch.dH3, m->batch.dH2, m->batch.dH1 };
	for (void* b : bufs)
		if (b) cudaFree(b);
	if (m->stream) cudaStreamDestroy(m->stream);
	delete m;
}

size_t srpGpuMlpParamCount(void) { return (size_t) kMlpParams; }

void srpGpuMlpGetParams(const SRPGpuMlp* m, float* out)
{
	cudaMemcpy(out, m->params, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost);
}

void srpGpuMlpSetParams(SRPGpuMlp* m, const float* in)
{
	cudaMemcpy(m->params, in, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
	m->packedValid = false;
}

void srpGpuMlpCapture(SRPGpuMlp* m, void (*target)(SRPFragmentShaderIn*, SRPFragmentShaderOut*), uint32_t every)
{
	L.capture = m;
	L.captureFs = target ? learnedShaderId((void*) target) : 0;
	L.captureEvery = every ? every : 1;
	if (m && L.captureFs != SRP_GPU_FS_MARBLE) {
		learnedError("srpGpuMlpCapture: only the marble shader (srpFsMarble) can be captured");
		L.capture = nullptr;
	}
}

size_t srpGpuMlpSampleCount(const SRPGpuMlp* m)
{
	unsigned long long n = 0;
	cudaDeviceSynchronize();
	cudaMemcpy(&n, m->count, sizeof n, cudaMemcpyDeviceToHost);
	return (size_t) (n < m->capacity ? n : m->capacity);
}

int srpGpuMlpAddSamples(SRPGpuMlp* m, const float* samples, size_t n)
{
	const size_t have = srpGpuMlpSampleCount(m);
	if (have + n > m->capacity) { learnedError("srpGpuMlpAddSamples: capacity exceeded"); return -1; }
	cudaMemcpy(m->samples + have * kSampleFloats, samples, n * kSampleFloats * sizeof(float), cudaMemcpyHostToDevice);
	const unsigned long long c = have + n;
	cudaMemcpy(m->count, &c, sizeof c, cudaMemcpyHostToDevice);
	return 0;
}

float srpGpuMlpTrain(SRPGpuMlp* m, int steps, int batch, float learningRate)
{
	const size_t n = srpGpuMlpSampleCount(m);
	if (!n || steps <= 0 || batch <= 0) { learnedError("srpGpuMlpTrain: no samples or no steps"); return -1.0f; }
	if (!reserveBatch(m, batch)) return -1.0f;
	cudaStream_t s = m->stream;
	cudaMemsetAsync(m->step, 0, sizeof(int), s);
	cudaMemsetAsync(m->adamM, 0, sizeof(float) * kMlpParams, s);
	cudaMemsetAsync(m->adamV, 0, sizeof(float) * kMlpParams, s);
	if (!m->graph || m->graphBatch != batch || m->graphSteps != steps || m->graphLr != learningRate ||
	    m->graphSamples != n) {
		if (m->graph) { cudaGraphExecDestroy(m->graph); m->graph = nullptr; }
		/* one training step, captured once and replayed */
		cudaGraph_t gr = nullptr;
		if (!ok(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "srpGpuMlpTrain capture")) return -1.0f;
		cudaMemsetAsync(m->grad, 0, sizeof(float) * kMlpParams, s);
		cudaMemsetAsync(m->sse, 0, sizeof(double), s);
		mlpGather(m->samples, (uint32_t) n, m->step, m->batch, batch, s);
		mlpForward(m->params, m->batch, batch, s);
		mlpBackward(m->params, m->grad, m->batch, batch, m->sse, s);
		mlpAdam(m->params, m->grad, m->adamM, m->adamV, m->step, steps, learningRate, s);
		if (!ok(cudaStreamEndCapture(s, &gr), "srpGpuMlpTrain capture") ||
		    !ok(cudaGraphInstantiate(&m->graph, gr, 0), "srpGpuMlpTrain instantiate")) {
			if (gr) cudaGraphDestroy(gr);
			return -1.0f;
		}
		cudaGraphDestroy(gr);
		m->graphBatch = batch;
		m->graphSteps = steps;
		m->graphLr = learningRate;
		m->graphSamples = n;   /* baked into the graph: a new count rebuilds it */
	}
	for (int i = 0; i < steps; ++i)
		if (!ok(cudaGraphLaunch(m->graph, s), "srpGpuMlpTrain")) return -1.0f;
	double sse = 0.0;
	cudaMemcpyAsync(&sse, m->sse, sizeof sse, cudaMemcpyDeviceToHost, s);
	if (!ok(cudaStreamSynchronize(s), "srpGpuMlpTrain")) return -1.0f;
	m->packedValid = false;
	return (float) (sse / ((double) batch * kMlpOut));
}

int srpGpuMlpEvaluate(SRPGpuMlp* m, const float* samples, size_t n, float* rgb, int tensorCores)
{
	if (!n) return 0;
	float* dSamples = nullptr;
	float* dOut = nullptr;
	if (!devAlloc(&dSamples, n * kSampleFloats, "srpGpuMlpEvaluate") || !devAlloc(&dOut, n * kMlpOut, "srpGpuMlpEvaluate"))
		return -1;
	cudaStream_t s = m->stream;
	cudaMemcpyAsync(dSamples, samples, n * kSampleFloats * sizeof(float), cudaMemcpyHostToDevice, s);
	int rc = 0;
	if (tensorCores) {
		unsigned err = 0;
		if (!packIfNeeded(m)) rc = -1;
		else {
			cudaMemsetAsync(m->tcErr, 0, sizeof(unsigned), s);
			mlpEvalTcgen05(dSamples, (int) n, m->packed5, m->bias, dOut, m->tcErr, s);
			cudaMemcpyAsync(&err, m->tcErr, sizeof err, cudaMemcpyDeviceToHost, s);
			if (!ok(cudaStreamSynchronize(s), "srpGpuMlpEvaluate")) rc = -1;
			else if (err) { learnedError("srpGpuMlpEvaluate: a tensor-core wait timed out"); rc = -1; }
		}
	} else {
		if (!reserveBatch(m, (int) n)) rc = -1;
		else {
			mlpEncode(dSamples, (int) n, m->batch, s);
			mlpForward(m->params, m->batch, (int) n, s);
			cudaMemcpyAsync(dOut, m->batch.Y, n * kMlpOut * sizeof(float), cudaMemcpyDeviceToDevice, s);
		}
	}
	if (rc == 0) {
		cudaMemcpyAsync(rgb, dOut, n * kMlpOut * sizeof(float), cudaMemcpyDeviceToHost, s);
		if (!ok(cudaStreamSynchronize(s), "srpGpuMlpEvaluate")) rc = -1;
	}
	cudaFree(dSamples);
	cudaFree(dOut);
	return rc;
}

int srpGpuMlpGradients(SRPGpuMlp* m, const float* samples, size_t n, float* grad, double* sse)
{
	if (!n) return 0;
	float* dSamples = nullptr;
	if (!devAlloc(&dSamples, n * kSampleFloats, "srpGpuMlpGradients") || !reserveBatch(m, (int) n)) return -1;
	cudaStream_t s = m->stream;
	std::vector<float> targets(n * kMlpOut);
	for (size_t i = 0; i < n; ++i)
		for (int k = 0; k < kMlpOut; ++k) targets[i * kMlpOut + k] = samples[i * kSampleFloats + 9 + k];
	cudaMemcpyAsync(dSamples, samples, n * kSampleFloats * sizeof(float), cudaMemcpyHostToDevice, s);
	cudaMemcpyAsync(m->batch.T, targets.data(), targets.size() * sizeof(float), cudaMemcpyHostToDevice, s);
	cudaMemsetAsync(m->grad, 0, sizeof(float) * kMlpParams, s);
	cudaMemsetAsync(m->sse, 0, sizeof(double), s);
	mlpEncode(dSamples, (int) n, m->batch, s);
	mlpForward(m->params, m->batch, (int) n, s);
	mlpBackward(m->params, m->grad, m->batch, (int) n, m->sse, s);
	cudaMemcpyAsync(grad, m->grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, s);
	cudaMemcpyAsync(sse, m->sse, sizeof(double), cudaMemcpyDeviceToHost, s);
	const int rc = ok(cudaStreamSynchronize(s), "srpGpuMlpGradients") ? 0 : -1;
	cudaFree(dSamples);
	return rc;
}

void srpGpuSetLearnedShading(void (*target)(SRPFragmentShaderIn*, SRPFragmentShaderOut*), SRPGpuMlp* m, float minPsnrDb,
                             uint32_t judgeEvery)
{
	L.net = m;
	L.targetFs = target ? learnedShaderId((void*) target) : 0;
	L.minPsnr = minPsnrDb;
	L.judgeEvery = judgeEvery ? judgeEvery : 1;
	if (m && L.targetFs != SRP_GPU_FS_MARBLE) {
		learnedError("srpGpuSetLearnedShading: only the marble shader (srpFsMarble) has a learned stand-in");
		L.net = nullptr;
	}
}

void srpGpuGetLearnedStats(SRPGpuLearnedStats* out) { *out = L.stats; }

void srpGpuResetLearnedStats(void) { L.stats = SRPGpuLearnedStats(); }

}  // extern "C"
