// axr_draw_mesh_noalloc: the draw of axr_draw_mesh for callers that cannot allocate
// device memory.
//
// The regular draw grows the context's scratch arena on demand (cudaMalloc after a stream
// synchronisation). Some callers cannot allow that: a renderer that records its frame
// into a CUDA graph (an allocation in the middle of a stream capture invalidates it), a
// real-time render loop that forbids allocator calls after start-up, or a host
// application that owns the device-memory budget and does not let plugins allocate. This
// entry point runs the same kernels with all of their scratch (vertex cache, large-
// triangle lists, resolve lists, work counters) in one file-scope device array of fixed
// size, so it calls no cudaMalloc, cudaFree or other allocating routine. The caller still
// creates the inputs (mesh, textures) and the output (framebuffer) beforehand.
//
// Limits: at most kNoAllocMaxVertices vertices, kNoAllocMaxFaces drawn faces and
// kNoAllocMaxPixels framebuffer pixels per call; larger draws are rejected with
// AXR_E_CAPACITY. The array (about 32 MiB) is reserved on every GPU that loads the library
// and stays reserved until the process exits.
//
// Set-up: the first call on each device looks up the array's device address with
// cudaGetSymbolAddress while that device is current; make that first call before any
// stream capture. The address is kept for the life of the process: after a
// cudaDeviceReset the library's module is loaded anew and the kept address is stale, so
// this entry point must not be used after one. All calls share the array and it keeps the
// last call's contents: each call clears the work counters it needs at zero, and two
// calls whose work overlaps on the GPU (different streams or contexts) race on the array.
//
// Reporting: after the draw, a one-thread kernel adds the array's error bits and (with
// statistics enabled on the context) its statistics to the context's counters, so
// axr_sync and axr_stats_read see this draw like any other; stage profiles
// (axr_profile_read) do not include it.
#include <cuda_runtime.h>

#include <mutex>

#include "api_internal.h"
#include "api_types.h"
#include "batch.h"

namespace {

constexpr uint32_t kNoAllocMaxVertices = 65536;
constexpr uint32_t kNoAllocMaxFaces = 65536;
constexpr uint32_t kNoAllocMaxPixels = 1024u * 1024u;
constexpr uint32_t kNoAllocMaxItems = 4u * kNoAllocMaxFaces;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffCounters = 0;
constexpr size_t kOffLarge = align256(kOffCounters + sizeof(axr::DevCounters));
constexpr size_t kOffItems = align256(kOffLarge + sizeof(axr::LargeTri) * kNoAllocMaxFaces);
constexpr size_t kOffVscreen = align256(kOffItems + sizeof(axr::LargeItem) * kNoAllocMaxItems);
constexpr size_t kOffVattr = align256(kOffVscreen + sizeof(float4) * kNoAllocMaxVertices);
constexpr size_t kOffShade = align256(kOffVattr + 4 * sizeof(float4) * kNoAllocMaxVertices);
constexpr size_t kOffClip = align256(kOffShade + sizeof(uint2) * kNoAllocMaxPixels);
constexpr size_t kOffRec = align256(kOffClip + sizeof(uint2) * kNoAllocMaxPixels);
constexpr size_t kNoAllocBytes = align256(kOffRec + sizeof(float4) * axr::kRecFloat4 * kNoAllocMaxFaces);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_device_base[kMaxDevices] = {};

// Device address of the array on `device` (current); looked up once per device.
cudaError_t scratch_base(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_device_base[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_device_base[device] = static_cast<unsigned char*>(ptr);
    }
    *out = g_device_base[device];
    return cudaSuccess;
}

axr_status noalloc_fail(axr_context* ctx, axr_status st, const std::string& msg) {
    ctx->error = msg;
    return st;
}

}  // namespace

extern "C" axr_status axr_draw_mesh_noalloc(axr_context* ctx, const axr_mesh* mesh, const float model[16]) {
    axr_internal::NvtxRange nvtx_range("axr_draw_mesh_noalloc");
    if (!ctx) return AXR_E_INVALID;
    if (!mesh || !model) return noalloc_fail(ctx, AXR_E_INVALID, "NULL mesh or model matrix");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->has_shader || !ctx->has_camera || !ctx->fb) return AXR_OK;  // as axr_draw_mesh
    const axr_framebuffer* fb = ctx->fb;
    const uint64_t pixels = (uint64_t)fb->width * (uint64_t)fb->height;
    if (mesh->num_vertices > kNoAllocMaxVertices || mesh->num_drawn > kNoAllocMaxFaces || pixels > kNoAllocMaxPixels)
        return noalloc_fail(ctx, AXR_E_CAPACITY,
                            "axr_draw_mesh_noalloc is limited to " + std::to_string(kNoAllocMaxVertices) +
                                " vertices, " + std::to_string(kNoAllocMaxFaces) + " faces and " +
                                std::to_string(kNoAllocMaxPixels) + " pixels; this draw has " +
                                std::to_string(mesh->num_vertices) + ", " + std::to_string(mesh->num_drawn) +
                                " and " + std::to_string(pixels));
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != ctx->device && cudaSetDevice(ctx->device) != cudaSuccess)
        return noalloc_fail(ctx, AXR_E_CUDA, "cannot make the context's device current");
    unsigned char* base = nullptr;
    cudaError_t e = scratch_base(ctx->device, &base);
    if (e == cudaSuccess) {
        using namespace axr;
        DrawParams p{};
        p.mesh = DevMesh{mesh->pos, mesh->nrm, mesh->tan, mesh->bit, mesh->uv, mesh->idx, mesh->groups,
                         mesh->materials, mesh->num_vertices, mesh->num_faces, mesh->num_groups, mesh->num_drawn};
        p.target = DevTarget{fb->color, fb->depth, fb->key, fb->tile_flag,
                             fb->width, fb->height, fb->tiles_x, fb->tiles_y};
        p.u = make_uniforms(ctx->camera, ctx->shader, model);
        DevCounters* counters = reinterpret_cast<DevCounters*>(base + kOffCounters);
        p.scratch = DevScratch{counters,
                               reinterpret_cast<LargeTri*>(base + kOffLarge),
                               reinterpret_cast<LargeItem*>(base + kOffItems),
                               reinterpret_cast<float4*>(base + kOffVscreen),
                               reinterpret_cast<float4*>(base + kOffVattr),
                               reinterpret_cast<uint2*>(base + kOffShade),
                               reinterpret_cast<uint2*>(base + kOffClip),
                               kNoAllocMaxFaces, kNoAllocMaxItems, kNoAllocMaxVertices, kNoAllocMaxPixels,
                               ctx->collect_stats, 0, nullptr, reinterpret_cast<float4*>(base + kOffRec)};
        p.small_max_pixels = ctx->small_max_pixels;
        // the array keeps the previous call's contents: start from zeroed counters
        e = cudaMemsetAsync(counters, 0, sizeof(DevCounters), ctx->stream);
        if (e == cudaSuccess) e = launch_draw(p, ctx->cfg, ctx->stream, &ctx->aux, nullptr, &ctx->launches);
        // the array's error bits and statistics into the context's counters
        if (e == cudaSuccess) e = launch_merge_counters(ctx->counters, counters, ctx->stream);
        if (e == cudaSuccess) ctx->launches += 1;
    }
    if (prev >= 0 && prev != ctx->device) cudaSetDevice(prev);
    if (e != cudaSuccess) return noalloc_fail(ctx, AXR_E_CUDA, std::string("axr_draw_mesh_noalloc: ") + cudaGetErrorString(e));
    return AXR_OK;
}
