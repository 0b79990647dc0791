/* What the draw paths of srp_api.cu and the learned-shading module
 * (srp_learned.cu) call on each other. */
#pragma once

#include <cuda_runtime.h>
#include "kernels.h"

namespace srpg {

/* Before a draw (nDraws = 1) or a multi-draw pass is enqueued: sets up the
 * fragment capture, and when the draw's shader is the learned target, turns
 * P into a learned-shaded draw (fsId = kFsLearned, judge cleared). Returns
 * true for a learned-shaded draw; P.judgeFs then holds the plain shader. */
bool learnedPrepare(DrawParams& P, int kind, bool late, uint32_t nDraws, cudaStream_t s);

/* After a learned-shaded draw or pass has been enqueued: waits for the
 * judge, records the statistics and sets redo[d] for every draw whose PSNR
 * is below the threshold (and, with redoDev, a device copy of redo).
 * When the network's kernel ran out of a bounded wait (kErrSpin in ctr's
 * errors), it reports that and marks every draw for redo. Returns the number
 * of draws marked. */
uint32_t learnedJudge(uint32_t nDraws, uint8_t* redo, const uint8_t** redoDev, cudaStream_t s,
                      const DeviceCounters* ctr);

/* srp_api.cu: error message through the user's callback, and the device id of
 * a host fragment shader (0 if it has none). */
void learnedError(const char* fmt, ...);
int learnedShaderId(void* fragmentShader);

}  // namespace srpg
