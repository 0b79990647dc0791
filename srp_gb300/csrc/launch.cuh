/* Kernel launches of the draw pipeline with programmatic dependent launch.
 *
 * A draw is a chain of dependent kernels on one stream (or one captured
 * graph). Launched with programmatic stream serialisation, the next kernel
 * of the chain is scheduled while the current one finishes, instead of after
 * it has drained; every kernel launched this way starts with gridDepSync(),
 * which waits until the preceding kernel has completed and its writes are
 * visible, so the ordering is that of plain launches. Only the launch latency
 * and the block scheduling overlap. */
#pragma once

#include <cuda_runtime.h>
#include <utility>

namespace srpg {

/* Waits for the preceding kernel of the stream (a no-op without one), then
 * allows the next kernel to be scheduled once every block of this grid has
 * started. Called first thing by every kernel launched with pdlLaunch. */
__device__ __forceinline__ void gridDepSync()
{
#if defined(__CUDA_ARCH__)
	asm volatile("griddepcontrol.wait;" ::: "memory");
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

template <typename... KArgs, typename... Args>
inline cudaError_t pdlLaunch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                             Args&&... args)
{
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = s;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace srpg
