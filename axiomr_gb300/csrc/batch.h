// Host launcher of the batched persistent kernel (batch.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch_types.h"
#include "kernels.h"

namespace axr {

// Resets the work counters and grid-barrier words, then launches the batch's draws (all
// of shader kind `shader`) in launch form `form`: kFormPersistent, one cooperative grid of
// (resident CTAs per SM) x num_sms CTAs running the four phases; kFormPhased, a clear
// kernel for the fully cleared draws and then four launches. `phase_events` (optional,
// 6 events, phased form only) are recorded around the five launches. `clear_late` (phased
// form, without phase events) runs the clear kernel after the large-triangle phase, right
// before the tile pass, instead of first. Adds the number of kernels launched to *launches.
cudaError_t launch_batch(int shader, const BatchParams& bp, int form, int num_sms, cudaStream_t stream,
                         cudaEvent_t* phase_events, uint64_t* launches, bool clear_late = false);

// Adds the statistics and error bits of `src` (a second launch set's counters) to `dst`
// and zeroes them in `src` (one thread).
cudaError_t launch_merge_counters(DevCounters* dst, DevCounters* src, cudaStream_t stream);

// Failure-path probe of the grid barrier: one CTA waits at a barrier the other never
// reaches; the bounded wait gives up after timeout_ns and sets the barrier error bit.
cudaError_t launch_barrier_probe(DevCounters* counters, unsigned long long timeout_ns, cudaStream_t stream);

}  // namespace axr
