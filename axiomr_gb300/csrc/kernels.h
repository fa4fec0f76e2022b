// Host-side launchers for the draw kernels (kernels.cu). All launches go to `stream`.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_types.h"

namespace axr {

// Side stream and events of a context: the clipped-winner resolve pass runs on the side
// stream, concurrently with the main shading pass (fork after the key scan, join after).
struct AuxStream {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};

struct LaunchConfig {
    int num_sms;
    int large_ctas_per_sm;
    int resolve_ctas_per_sm;
    // no vertex of the draw can lie outside or on a clip plane (checked on the host from the
    // mesh's bounding sphere): no triangle is clipped, so the clipped-winner pass is not run
    bool clip_free = false;
};

// One draw: geometry (transform, clip, cull, setup, small-triangle raster) -> large
// triangle tile raster -> per-tile resolve and shading into the framebuffer.
// `stage_events` (optional, kStageEvents events) are recorded before the first kernel and
// after each of the six (vertex, geometry, large, scan, shade, clipped). Adds the number
// of kernels launched to *launches.
constexpr int kStageEvents = 7;
cudaError_t launch_draw(const DrawParams& p, const LaunchConfig& cfg, cudaStream_t stream, const AuxStream* aux,
                        cudaEvent_t* stage_events, uint64_t* launches);

cudaError_t launch_clear(uint32_t* color, float* depth, size_t pixels, uint32_t bgra, float depth_value,
                         bool do_color, bool do_depth, cudaStream_t stream);
cudaError_t launch_fill_u64(unsigned long long* dst, size_t n, unsigned long long v, cudaStream_t stream);
// float3 (packed) -> float4 (x, y, z, 0)
cudaError_t launch_pack3(const float* src, float4* dst, uint32_t n, cudaStream_t stream);
// Bounds of pos[0, n) into *out (device); the box centre and squared radius follow the
// host's mesh_bounds operation for operation.
cudaError_t launch_mesh_bounds(const float4* pos, uint32_t n, MeshBounds* out, cudaStream_t stream);
// The float an order-preserving integer of launch_mesh_bounds stands for.
float mesh_bounds_float(uint32_t ord);
// RGBA8 bytes of a uint32 array (no conversion needed; provided for symmetry)

// Stage dump for parity tests: every triangle that survives clip + cull, unordered, as
// (tag, screen x0 y0 x1 y1 x2 y2, ndcZ0..2, minX, minY, maxX, maxY) = 14 words.
cudaError_t launch_debug_triangles(const DrawParams& p, float* out, uint32_t* count, uint32_t capacity,
                                   cudaStream_t stream);
cudaError_t launch_debug_sample(DevTexture tex, const float2* uv, float4* out, uint32_t n, cudaStream_t stream);

}  // namespace axr
