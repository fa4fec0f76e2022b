// Host launcher of the batched persistent kernel (batch.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch_types.h"

namespace axr {

// Resets the work counters and grid-barrier words, then launches one cooperative grid of
// (resident CTAs per SM) x num_sms CTAs running the four phases over the batch's draws,
// which must all use shader kind `shader`. Adds the number of kernels launched to
// *launches.
cudaError_t launch_batch(int shader, const BatchParams& bp, int num_sms, cudaStream_t stream, uint64_t* launches);

}  // namespace axr
