// Packed read-back: the colour planes of many framebuffers gathered into one device
// buffer, image after image, so that one large copy brings them all to the host (one
// copy of this kind reaches the device-to-host link rate; hundreds of per-plane copies do
// not). Two formats: the planes as stored (BGRA8, framebuffer row 0 first = the bottom of
// the picture) or RGB8 with the top row first, the picture the reference's window shows
// (Window::present, src/window.cpp:70-84, through a bottom-up DIB that ignores alpha).
#include <cuda_runtime.h>

#include "api_internal.h"
#include "api_types.h"

namespace axr {

struct PackedParams {
    const PackedImage* images;
    uint8_t* dst;
    uint32_t count, rgb;
    unsigned long long pixels;
};

__global__ void __launch_bounds__(256) packed_kernel(const __grid_constant__ PackedParams p) {
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long g = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; g < p.pixels; g += stride) {
        uint32_t lo = 0, hi = p.count;  // the image holding pixel g
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (p.images[mid].first <= g) lo = mid; else hi = mid;
        }
        const PackedImage& im = p.images[lo];
        const unsigned long long k = g - im.first;
        const uint32_t v = __ldcs(im.color + k);
        if (!p.rgb) {
            reinterpret_cast<uint32_t*>(p.dst + im.out)[k] = v;
        } else {
            const uint32_t y = (uint32_t)(k / im.width), x = (uint32_t)(k - (unsigned long long)y * im.width);
            uint8_t* o = p.dst + im.out + 3ull * ((unsigned long long)(im.height - 1 - y) * im.width + x);
            o[0] = (uint8_t)(v >> 16);  // R
            o[1] = (uint8_t)(v >> 8);   // G
            o[2] = (uint8_t)v;          // B
        }
    }
}

}  // namespace axr

namespace axr_internal {

cudaError_t launch_packed(const axr::PackedImage* images_dev, uint32_t count, unsigned long long pixels, bool rgb,
                          uint8_t* dst, int num_sms, cudaStream_t stream) {
    axr::PackedParams p{images_dev, dst, count, rgb ? 1u : 0u, pixels};
    const unsigned long long want = (pixels + 255) / 256;
    const unsigned blocks = (unsigned)(want < (unsigned long long)num_sms * 16 ? (want ? want : 1) : num_sms * 16ull);
    axr::packed_kernel<<<blocks, 256, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace axr_internal
