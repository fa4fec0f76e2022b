// Helpers shared by the files that implement C ABI entry points (api.cpp, batch_api.cpp):
// error reporting into the context, device selection and allocation wrappers.
#pragma once
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include "api_types.h"

namespace axr {
// One colour plane of a packed read-back (csrc/readback.cu).
struct PackedImage {
    const uint32_t* color;
    unsigned long long out;    // byte offset of the image in the packed buffer
    uint32_t width, height;
    unsigned long long first;  // first pixel of the image in the call's pixel range
};
}

namespace axr_internal {

// NVTX range over a host entry point, so that a timeline tool shows the library's calls
// beside their kernels (a few nanoseconds when no tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Record a formatted message as the context's last error (or the thread's, without a
// context) and return `st`.
axr_status fail(axr_context* ctx, axr_status st, const char* fmt, ...);
// AXR_E_OOM for an allocation failure, AXR_E_CUDA otherwise.
axr_status cuda_fail(axr_context* ctx, cudaError_t e, const char* what);
void dfree(void* p);
// Fill fb->color_map / depth_map for TMA tile stores (sets fb->tma; false when the row
// pitch is not a multiple of 16 bytes or the driver lacks the entry point).
void encode_framebuffer_maps(axr_framebuffer* fb);
// Bounding sphere (box centre, largest distance) of n float3 positions.
void mesh_bounds(const float* pos, uint32_t n, float center[3], float* radius);
// Waits for and takes the device-computed bounds of the last axr_mesh_update, if any.
void mesh_sync_bounds(const axr_mesh* m);
// Release a batch's device memory (the caller synchronises first).
void free_batch(axr_batch* b);
// Release a batch's pinned staging and its events (the caller synchronises first).
void free_batch_staging(axr_batch* b);
// Plan `count` draws into `b` / launch a planned batch on the context stream (the caller
// holds ctx->mu; axr_batch_create / axr_batch_launch without the locking).
axr_status batch_plan(axr_context* ctx, const axr_draw_desc* draws, int32_t count, axr_batch* b, bool async);
axr_status batch_launch(axr_context* ctx, const axr_batch* b);
// The gather of colour planes behind axr_readback_start_packed (csrc/readback.cu):
// `images_dev` (device) lists each plane, its byte offset in dst and its first pixel in
// the call's range of `pixels`; rgb: RGB8 top row first, else BGRA8 as stored.
cudaError_t launch_packed(const axr::PackedImage* images_dev, uint32_t count, unsigned long long pixels, bool rgb,
                          uint8_t* dst, int num_sms, cudaStream_t stream);
// Release the PNG encoder's scratch (the caller synchronises first).
void free_png(axr_context* ctx);
// PNG batches for the serving loop, without blocking: create / release; enqueue an encode
// (the caller holds ctx->mu); query whether the encode and its size copy are done
// (cudaErrorNotReady while not); then file i's device address and size (0: overflow).
axr_status png_batch_create(axr_context* ctx, axr_png_batch** out);
void png_batch_release(axr_png_batch* b);
axr_status png_batch_encode_locked(axr_context* ctx, axr_png_batch* b, int32_t count,
                                   const axr_framebuffer* const* fbs, uint32_t channels);
cudaError_t png_batch_query(const axr_png_batch* b);
void png_batch_file(const axr_png_batch* b, int32_t i, const void** dev, uint64_t* size);

// Bin parameters within their documented ranges (capacity and shape 0 allowed only where
// they mean "chosen per draw").
inline bool valid_bin_params(const axr_bin_params& b, bool allow_auto) {
    auto pow2_tiles = [](int32_t v) { return v == 1 || v == 2 || v == 4 || v == 8; };
    const bool cap_ok = (allow_auto && b.capacity == 0) || (b.capacity >= 16 && b.capacity <= 65536);
    const int32_t ty = b.tiles_y ? b.tiles_y : (b.tiles_x ? 8 / b.tiles_x : 1);
    const bool shape_ok = (allow_auto && b.tiles_x == 0) ||
                          (pow2_tiles(b.tiles_x) && pow2_tiles(ty) && b.tiles_x * ty <= 8);
    return cap_ok && shape_ok && b.thread_pixels >= 1 && b.thread_pixels <= 2048;
}

// Tiles across and down of a bin from valid parameters with a fixed shape.
inline void bin_shape(const axr_bin_params& b, uint8_t* tw, uint8_t* th) {
    *tw = (uint8_t)b.tiles_x;
    *th = (uint8_t)(b.tiles_y ? b.tiles_y : 8 / b.tiles_x);
}

template <class T>
cudaError_t dmalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
}

// Makes `dev` current for the scope and restores the previous device.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace axr_internal

#define AXR_CUDA(ctx, call)                                                      \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) return axr_internal::cuda_fail((ctx), e_, #call); \
    } while (0)
