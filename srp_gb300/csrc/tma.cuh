/* Inline PTX for tensor-memory-access (TMA) copies of framebuffer tiles
 * between global and shared memory: 2-D tiled loads completed on an
 * mbarrier, and 2-D tiled stores committed as bulk groups.
 *
 * A tile copy moves an 8 x 8 box of 32-bit pixels (32 bytes a row) of a
 * plane described by a CUtensorMap that the host encodes for the plane's
 * width, height and row pitch (a multiple of 16 bytes). The box starts at
 * pixel x = 8 * tile column, so its first byte is 16-byte aligned; parts of
 * a box beyond the plane's edge read as zero and are not written.
 *
 * Every wait is bounded (mbarWait of tc5.cuh); the caller records a timeout
 * and returns. */
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "tc5.cuh"

namespace srpg {

/* The kernel-parameter copy of a tensor map, as the generic address PTX
 * takes (a __grid_constant__ parameter's address). */
__device__ __forceinline__ uint64_t tmaMapAddr(const CUtensorMap* m) { return (uint64_t) (uintptr_t) m; }

/* Makes an initialised mbarrier visible to the tensor-copy unit. */
__device__ __forceinline__ void fenceMbarInit()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

/* Arrive on the mbarrier and expect `bytes` more of asynchronous copies. */
__device__ __forceinline__ void mbarArriveExpectTx(uint32_t mbar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

/* Tile (x, y) of the plane -> shared memory at dst (128-byte aligned); the
 * mbarrier completes when its bytes have landed. */
__device__ __forceinline__ void tmaLoad2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t mbar)
{
	asm volatile(
	    "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
	    ::"r"(dst), "l"(tmaMapAddr(map)), "r"(x), "r"(y), "r"(mbar)
	    : "memory");
}

/* Shared memory at src -> tile (x, y) of the plane, in the current bulk
 * group. The threads' writes to src must be fenced (fenceProxyAsync) and
 * synchronised with the issuing thread first. */
__device__ __forceinline__ void tmaStore2d(const CUtensorMap* map, int x, int y, uint32_t src)
{
	asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
	             ::"l"(tmaMapAddr(map)), "r"(x), "r"(y), "r"(src)
	             : "memory");
}

__device__ __forceinline__ void bulkCommit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

/* Wait until the committed stores have read their shared-memory sources
 * (the shared memory may then be reused or released). */
__device__ __forceinline__ void bulkWaitRead() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

}  // namespace srpg
