/* Inline PTX for the 5th-generation tensor cores (tcgen05) and their
 * shared-memory operands, as used by the learned-shading network.
 *
 * Operands are bf16 matrices in the canonical K-major layout without
 * swizzling: 8-row x 16-byte "core matrices"; element (r, k) of a matrix with
 * K columns sits at (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
 * bytes, SBO = K / 8 * 128. One MMA consumes K = 16 (two core matrices along
 * K), so step s of a matrix starts 256 * s bytes further on.
 *
 * Every wait on an mbarrier is bounded: after kTcSpinLimit polls it gives up
 * and reports failure, so that a kernel can record an error, release its
 * tensor memory and return. */
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace srpg {

__device__ __forceinline__ uint32_t packBf16(float lo, float hi)
{
	const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
	return *(const uint32_t*) &v;
}

constexpr unsigned kTcSpinLimit = 1u << 24;

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t) __cvta_generic_to_shared(p); }

/* byte offset of element (r, k) of a K-column bf16 operand */
__device__ __forceinline__ uint32_t tcOffset(int r, int k, int K)
{
	return (uint32_t) ((r >> 3) * (K / 8 * 128) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

/* Shared-memory matrix descriptor: start address, leading-dimension byte
 * offset (between core matrices along K), stride byte offset (between
 * 8-row groups), descriptor version 1, no swizzle. */
__device__ __forceinline__ uint64_t tcDesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
	return (uint64_t) ((addr >> 4) & 0x3FFFu) | (uint64_t) ((lbo >> 4) & 0x3FFFu) << 16 |
	       (uint64_t) ((sbo >> 4) & 0x3FFFu) << 32 | (uint64_t) 1 << 46;
}

/* Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
 * K-major, M x N. */
__host__ __device__ constexpr uint32_t tcIdescBf16(int M, int N)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (N >> 3) << 17) | ((uint32_t) (M >> 4) << 24);
}

__device__ __forceinline__ void tcAlloc(uint32_t slotAddr, uint32_t cols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slotAddr), "r"(cols));
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tcDealloc(uint32_t taddr, uint32_t cols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols));
}

__device__ __forceinline__ void tcMma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t accumulate)
{
	asm volatile(
	    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dTmem),
	    "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tcCommit(uint32_t mbarAddr)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbarAddr)
	             : "memory");
}

__device__ __forceinline__ void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
/* generic-proxy shared-memory writes become visible to the tensor cores */
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbarInit(uint32_t addr, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}

/* Bounded wait for the phase with the given parity to complete: at most
 * `limit` polls (0 = kTcSpinLimit). */
__device__ __forceinline__ bool mbarWait(uint32_t addr, uint32_t parity, uint32_t limit = 0)
{
	const unsigned polls = limit ? limit : kTcSpinLimit;
	for (unsigned i = 0; i < polls; ++i) {
		uint32_t done;
		asm volatile(
		    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		    "selp.u32 %0, 1, 0, p;\n\t}\n"
		    : "=r"(done)
		    : "r"(addr), "r"(parity)
		    : "memory");
		if (done) return true;
	}
	return false;
}

/* Named barrier `id` over `threads` threads (a multiple of 32): plain, and
 * with an OR or AND of a predicate over the participants. */
__device__ __forceinline__ void namedSync(uint32_t id, uint32_t threads)
{
	asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

__device__ __forceinline__ bool namedSyncOr(uint32_t id, uint32_t threads, bool p)
{
	uint32_t r;
	asm volatile(
	    "{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\tbar.red.or.pred b, %2, %3, a;\n\t"
	    "selp.u32 %0, 1, 0, b;\n\t}\n"
	    : "=r"(r)
	    : "r"((uint32_t) p), "r"(id), "r"(threads)
	    : "memory");
	return r != 0;
}

__device__ __forceinline__ bool namedSyncAnd(uint32_t id, uint32_t threads, bool p)
{
	uint32_t r;
	asm volatile(
	    "{\n\t.reg .pred a, b;\n\tsetp.ne.u32 a, %1, 0;\n\tbar.red.and.pred b, %2, %3, a;\n\t"
	    "selp.u32 %0, 1, 0, b;\n\t}\n"
	    : "=r"(r)
	    : "r"((uint32_t) p), "r"(id), "r"(threads)
	    : "memory");
	return r != 0;
}

/* 16 consecutive fp32 columns of this thread's TMEM lane. */
__device__ __forceinline__ void tcLoad16(uint32_t taddr, float v[16])
{
	uint32_t r[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

/* One layer's MMAs, issued by one thread: D[128 x N] = A[128 x K] B^T with
 * A and B in the canonical layout (K a multiple of 16; N 64 or 16). */
__device__ __forceinline__ void tcLayer(uint32_t tmem, uint32_t aAddr, uint32_t bAddr, int K, int N)
{
	const uint32_t sbo = (uint32_t) (K / 8 * 128);
	const uint32_t idesc = N == 64 ? tcIdescBf16(128, 64) : tcIdescBf16(128, 16);
	for (int s = 0; s < K / 16; ++s)
		tcMma(tmem, tcDesc(aAddr + 256u * s, 128, sbo), tcDesc(bAddr + 256u * s, 128, sbo), idesc, s > 0 ? 1u : 0u);
}

}  // namespace srpg
