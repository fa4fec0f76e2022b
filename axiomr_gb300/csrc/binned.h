// Host launchers of the binned form (binned.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch_types.h"
#include "kernels.h"

namespace axr {

// Kernel parameters of one binned draw. flags: kBatchTma when the tensor maps are valid,
// kBatchClearColor / kBatchClearDepth to fuse the clear of a plane into the bin pass (the
// per-draw entry point clears nothing: the draw merges into the framebuffer as it is).
struct alignas(64) SoloBinned {
    TensorMap128 color_map, depth_map;
    DrawParams p;
    BinSet bins;
    uint32_t flags;
    uint32_t clear_bgra;
    float clear_depth;
    uint32_t pad_;
};

// Bin geometry of a framebuffer for a bin of tw x th tiles (tw * th == kBinTiles).
inline void bin_geometry(int tiles_x, int tiles_y, int tw, int th, uint16_t* bins_x, uint16_t* bins_y) {
    *bins_x = (uint16_t)((tiles_x + tw - 1) / tw);
    *bins_y = (uint16_t)((tiles_y + th - 1) / th);
}

// One draw: zeroes the draw's counters and the bin counts, then three launches (vertices,
// faces, bins). `stage_events` (optional, kStageEvents events): recorded before the first
// kernel, after the vertex kernel, three times after the face kernel (the keyed form's
// geometry, large-triangle and scan stages) and twice after the bin kernel (its shading
// and clipped stages), so the profile reports the faces as geometry and the bin pass as
// shading. Adds the kernels launched to *launches.
cudaError_t launch_draw_binned(const SoloBinned& sb, cudaStream_t stream, cudaEvent_t* stage_events,
                               uint64_t* launches);

// One launch set of a batch in the binned form: counters and bin counts zeroed, then the
// vertex, face and bin launches over its units. `phase_events` (optional, 6 events) are
// recorded so that the phase profile reports vertices, faces and bins (clear and
// large-triangle phases empty).
cudaError_t launch_batch_binned(int shader, const BatchParams& bp, cudaStream_t stream, cudaEvent_t* phase_events,
                                uint64_t* launches);

}  // namespace axr
