// FP32 issue-peak microbenchmark: the denominator of the fragment-ALU side of the frame
// roofline (fragment ALU operations over FP32 issue peak). Every thread runs eight
// independent fused multiply-add chains (two flops per FMA), so the SMs' FP32 pipes stay
// full; the achieved rate over a fully occupied grid is the measured peak at the clocks
// the GPU is running.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "api_internal.h"
#include "api_types.h"

namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;

__global__ void __launch_bounds__(256) fma_chains_kernel(float* sink, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int k = 0; k < kChains; ++k) x[k] = __fmaf_rn(x[k], a, b);
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) acc += x[k];
    if (acc == 1234.5f) sink[blockIdx.x] = acc;  // keeps the chains live; practically never taken
}

}  // namespace

using namespace axr_internal;

extern "C" axr_status axr_measure_fp32_peak(axr_context* ctx, double* tflops) {
    if (!ctx || !tflops) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    int per_sm = 0;
    AXR_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_chains_kernel, 256, 0));
    const unsigned grid = (unsigned)(std::max(1, per_sm) * ctx->cfg.num_sms * 4);
    const int iters = 256;
    float* sink = nullptr;
    AXR_CUDA(ctx, cudaMallocAsync(&sink, sizeof(float) * grid, ctx->stream));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    AXR_CUDA(ctx, cudaEventCreate(&e0));
    AXR_CUDA(ctx, cudaEventCreate(&e1));
    double best = 0.0;
    cudaError_t e = cudaSuccess;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
        e = cudaEventRecord(e0, ctx->stream);
        if (e == cudaSuccess) fma_chains_kernel<<<grid, 256, 0, ctx->stream>>>(sink, iters, 0.999f, 1e-4f);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * kChains * kUnroll * (double)iters * 256.0 * grid;
        if (e == cudaSuccess && rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
        ++ctx->launches;
    }
    cudaFreeAsync(sink, ctx->stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fp32 peak");
    *tflops = best;
    return AXR_OK;
}
