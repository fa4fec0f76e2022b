// Definitions behind the C ABI's opaque handles (include/axr.h), shared by the .cu/.cpp
// files that implement entry points, plus the per-draw uniform computation.
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "axr.h"
#include "batch_types.h"
#include "binned.h"
#include "device_types.h"
#include "hostmath.h"
#include "kernels.h"

namespace axr_internal {
struct PngState;  // scratch of the PNG encoder (encode.cu)
}

using axr::DevCounters;
using axr::DevGroup;
using axr::DevMaterial;
using axr::LargeItem;
using axr::LargeTri;
using axr::LaunchConfig;

struct axr_texture {
    uint32_t* texels = nullptr;
    int32_t width = 0, height = 0;
    int device = 0;
};

struct axr_mesh {
    float4* pos = nullptr;
    float4* nrm = nullptr;
    float4* tan = nullptr;
    float4* bit = nullptr;
    float2* uv = nullptr;
    uint32_t* idx = nullptr;
    DevGroup* groups = nullptr;
    DevMaterial* materials = nullptr;
    float* staging = nullptr;  // packed float3 upload area for updates
    uint32_t num_vertices = 0, num_faces = 0, num_groups = 0, num_materials = 0, num_drawn = 0;
    int device = 0;
    // bounding sphere of the positions (batch planning): from the host arrays at creation;
    // after axr_mesh_update computed on the device on the update's stream and copied into
    // bounds_host behind bounds_ready (read through mesh_sync_bounds)
    mutable float bound_center[3] = {0.f, 0.f, 0.f};
    mutable float bound_radius = 0.f;
    mutable bool bounds_pending = false;
    axr::MeshBounds* bounds_dev = nullptr;
    axr::MeshBounds* bounds_host = nullptr;  // pinned
    cudaEvent_t bounds_ready = nullptr;
};

struct axr_framebuffer {
    uint32_t* color = nullptr;
    float* depth = nullptr;
    unsigned long long* key = nullptr;
    uint32_t* tile_flag = nullptr;
    int32_t width = 0, height = 0, tiles_x = 0, tiles_y = 0;
    int device = 0;
    // TMA descriptors of the colour and depth planes (16x16 boxes), valid when tma is set
    // (the row pitch must be a multiple of 16 bytes: width % 4 == 0)
    axr::TensorMap128 color_map{}, depth_map{};
    bool tma = false;
};

// A planned batch (batch_api.cpp): the draw table and scratch in one device allocation,
// and one launch description per shader kind present.
struct axr_batch {
    struct Launch {
        int shader;
        int set;  // launch set: 0 on the context stream, 1 on the batch side stream
        axr::BatchParams params;
    };
    int device = 0;
    void* dev = nullptr;
    size_t bytes = 0;
    std::vector<Launch> launches;
    int sets = 1;                               // launch sets (phased form of a large batch: 2)
    axr::DevCounters* set_counters = nullptr;  // counters of launch set 1 (in `dev`)
    int form = 0;  // axr::kForm*
    uint32_t count = 0;
    uint64_t vertices = 0, faces = 0, pixels = 0, tiles = 0;
    // pinned staging of the draw and unit tables for uploads on the context stream; two,
    // used in turn, so that planning the next batch does not wait for the last upload
    void* stage[2] = {};
    size_t stage_bytes[2] = {};
    cudaEvent_t stage_done[2] = {};
    int stage_next = 0;
};

struct axr_graph {
    cudaGraphExec_t exec = nullptr;
    int device = 0;
};

struct axr_context {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    axr::AuxStream aux{};  // side stream + fork/join events for the clipped-winner pass
    axr::AuxStream batch_side{};  // second launch set of a split batch (normal priority)
    // read-back streams of axr_framebuffers_read_async (created on first use): copies of many
    // framebuffers are spread over them so that several copy engines run at once
    static constexpr int kCopyStreams = 4;
    cudaStream_t copy_stream[kCopyStreams] = {};
    cudaEvent_t copy_fork = nullptr, copy_join[kCopyStreams] = {};
    LaunchConfig cfg{};
    std::mutex mu;
    std::string error;
    bool capturing = false;
    // pipeline state (Pipeline::m_Shader, m_Camera, m_Framebuffer)
    bool has_shader = false, has_camera = false;
    axr_shader_desc shader{};
    axr_camera_desc camera{};
    axr_framebuffer* fb = nullptr;
    // device scratch arena
    DevCounters* counters = nullptr;
    LargeTri* large = nullptr;
    LargeItem* items = nullptr;
    float4* vscreen = nullptr;
    float4* vattr = nullptr;
    uint2* shade = nullptr;
    uint2* clip_px = nullptr;
    float4* rec = nullptr;  // shading records (kRecFloat4 per face in draw order)
    uint32_t large_cap = 0, item_cap = 0, vcap = 0, px_cap = 0, rec_cap = 0;
    int collect_stats = 0;
    int small_max_pixels = 64;
    // batched form: per density class, the largest pixel box rasterised per thread
    // (autotuned), and the reusable plan of axr_draw_batch
    int32_t tune_small[AXR_TUNE_CLASSES] = {64, 64, 64, 64, 64, 64};
    // binned batched form: bin parameters per density class (autotuned)
    axr_bin_params tune_bin[AXR_TUNE_CLASSES] = {{256, 4, 64, 2}, {256, 4, 64, 2}, {256, 4, 64, 2},
                                                 {256, 4, 64, 2}, {256, 4, 64, 2}, {256, 4, 64, 2}};
    // binned per-draw form (axr_draw_mesh): its parameters and scratch: the bin counters
    // followed by the bin counts, the bins' entries and the clipped-triangle records
    int draw_form = AXR_DRAW_KEYED;
    axr_bin_params bin_params{0, 0, 64, 0};
    axr::BinCounters* bin_mem = nullptr;
    uint32_t* bin_entries = nullptr;
    float4* bin_crec = nullptr;
    uint32_t bin_count_cap = 0, crec_cap = 0;
    size_t bin_entry_cap = 0;
    axr_batch* oneshot = nullptr;
    axr::BatchProfile* batch_prof = nullptr;  // device-side phase timing of persistent launches
    int batch_form = axr::kFormPhased;        // launch form of batches planned next
    std::vector<cudaEvent_t> batch_events;     // phase events of phased launches (6 per launch)
    size_t batch_events_used = 0;
    // profiling: per-draw stage events (4 per draw), reused across reads
    bool profile = false;
    std::vector<cudaEvent_t> event_pool;
    size_t events_used = 0;
    uint64_t launches = 0;
    axr_internal::PngState* png = nullptr;
};

namespace axr {

// Uniforms the draw kernels read: mvp = viewProj * modelMatrix (src/tiled_pipeline.cpp:149)
// in the kernels' association order, the Flat shader's normal matrix, eye and lights.
inline DevUniforms make_uniforms(const axr_camera_desc& cam, const axr_shader_desc& sh, const float* model) {
    DevUniforms u{};
    host::M4 vp = host::load(cam.view_proj);
    host::M4 mm = host::load(model);
    host::M4 mvp = host::mul(vp, mm);  // viewProj * modelMatrix (src/tiled_pipeline.cpp:149)
    std::memcpy(u.mvp, mvp.m, sizeof(u.mvp));
    std::memcpy(u.model, model, sizeof(u.model));
    if (sh.kind == AXR_SHADER_FLAT) host::normal_matrix(mm, u.normal_mat);
    std::memcpy(u.cam_pos, cam.position, sizeof(u.cam_pos));
    std::memcpy(u.light_dir, sh.light_direction, sizeof(u.light_dir));
    std::memcpy(u.light_color, sh.light_color, sizeof(u.light_color));
    u.shader = sh.kind;
    return u;
}

}  // namespace axr
