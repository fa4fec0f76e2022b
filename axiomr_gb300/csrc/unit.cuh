// Work units of the batched forms: a unit names a draw of the batch and a unit index inside
// it (UnitRef); a CTA copies that draw's parameters into shared memory before its work.
#pragma once
#include <cuda_runtime.h>

#include "batch_types.h"

namespace axr {
namespace {

struct UnitInfo {
    uint32_t draw;   // index into the batch
    uint32_t local;  // unit index inside the draw
    uint32_t flags, clear_bgra;
    float clear_depth;
    uint32_t pad_[3];
};

// Warp 0 copies the parameters of work unit u's draw into shared memory.
__device__ __forceinline__ void stage_unit(const BatchParams& bp, uint32_t u, DrawParams* dst, UnitInfo* info) {
    if (threadIdx.x < 32) {
        const uint2 r = __ldg(reinterpret_cast<const uint2*>(bp.units) + u);
        const BatchDraw* bd = &bp.draws[r.x];
        const uint4* src = reinterpret_cast<const uint4*>(&bd->p);
        uint4* out = reinterpret_cast<uint4*>(dst);
        for (int k = (int)threadIdx.x; k < (int)(sizeof(DrawParams) / 16); k += 32) out[k] = __ldg(src + k);
        if (threadIdx.x == 0)
            *info = UnitInfo{r.x, r.y, __ldg(&bd->flags), __ldg(&bd->clear_bgra), __ldg(&bd->clear_depth), {0, 0, 0}};
    }
}

}  // namespace
}  // namespace axr
