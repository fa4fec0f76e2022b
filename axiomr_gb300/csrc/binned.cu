// Kernels of the binned form (device code in binned.cuh): a single draw (three launches:
// vertices, faces, bins) and a batch of draws (the same three launches over the work units
// of every draw of a launch set, each CTA staging its unit's draw parameters).
#include <cuda_runtime.h>

#include "binned.cuh"
#include "binned.h"
#include "unit.cuh"

namespace axr {
namespace {

constexpr int kBlock = 256;

// Resident CTAs per SM the bin kernel is compiled for. 4 gives it 64 registers (68 bytes
// of spills); 5 (48 registers, 256 bytes of spills) measured 6% slower on the 512-draw
// batch, its spilled locals going to L2 and DRAM beside the tile stores.
#ifndef AXR_BIN_MIN_BLOCKS
#define AXR_BIN_MIN_BLOCKS 4
#endif
#ifndef AXR_BIN_FACE_MIN_BLOCKS
#define AXR_BIN_FACE_MIN_BLOCKS 4
#endif

// ---- single draw
template <int S>
__global__ void __launch_bounds__(kBlock) solo_vertex_kernel(const __grid_constant__ SoloBinned sb) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < sb.p.mesh.num_vertices) vertex_one<S>(sb.p, i);
}

__global__ void __launch_bounds__(kBlock, AXR_BIN_FACE_MIN_BLOCKS) solo_face_kernel(const __grid_constant__ SoloBinned sb) {
    const uint32_t o = blockIdx.x * kBlock + threadIdx.x;
    bin_face(sb.p, sb.bins, o, o < sb.p.mesh.num_drawn, sb.p.scratch.counters, sb.p.scratch.collect_stats != 0);
}

template <int S>
__global__ void __launch_bounds__(kBinThreads, AXR_BIN_MIN_BLOCKS) solo_bin_kernel(const __grid_constant__ SoloBinned sb) {
    __shared__ __align__(128) BinSmem sm;
    bin_tile<S>(sb.p, sb.bins, blockIdx.x, &sb.color_map, &sb.depth_map, sb.flags, sb.clear_bgra, sb.clear_depth, sm,
                sb.p.scratch.counters, sb.p.scratch.collect_stats != 0);
}

// ---- batch: face units and bin units of every draw of a launch set
__global__ void __launch_bounds__(kBlock, AXR_BIN_FACE_MIN_BLOCKS) batch_bin_face_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p;
    __shared__ UnitInfo s_u;
    stage_unit(bp, bp.vert_units + blockIdx.x, &s_p, &s_u);
    __syncthreads();
    const uint32_t o = s_u.local * kFaceUnit + threadIdx.x;
    bin_face(s_p, bp.bins, o, o < s_p.mesh.num_drawn, bp.counters, bp.collect_stats != 0);
}

template <int S>
__global__ void __launch_bounds__(kBinThreads, AXR_BIN_MIN_BLOCKS) batch_bin_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p;
    __shared__ UnitInfo s_u;
    __shared__ __align__(128) BinSmem sm;
    stage_unit(bp, bp.vert_units + bp.face_units + blockIdx.x, &s_p, &s_u);
    __syncthreads();
    const BatchDraw* bd = &bp.draws[s_u.draw];
    bin_tile<S>(s_p, bp.bins, s_u.local, &bd->color_map, &bd->depth_map, s_u.flags, s_u.clear_bgra, s_u.clear_depth, sm,
                bp.counters, bp.collect_stats != 0);
}

template <int S>
__global__ void __launch_bounds__(kBlock) batch_bin_vertex_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p;
    __shared__ UnitInfo s_u;
    stage_unit(bp, blockIdx.x, &s_p, &s_u);
    __syncthreads();
    const uint32_t i = s_u.local * kVertUnit + threadIdx.x;
    if (i < s_p.mesh.num_vertices) vertex_one<S>(s_p, i);
}

unsigned blocks_for(size_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

template <int S>
cudaError_t launch_solo_s(const SoloBinned& sb, cudaStream_t stream, cudaEvent_t* ev, uint64_t* launches) {
    cudaError_t e;
    auto mark = [&](int k) { return ev ? cudaEventRecord(ev[k], stream) : cudaSuccess; };
    const size_t bin_bytes = sizeof(BinCounters) + sizeof(uint32_t) * (size_t)sb.bins.nbins;
    if ((e = cudaMemsetAsync(sb.p.scratch.counters, 0, kCountersReset, stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(sb.bins.counters, 0, bin_bytes, stream)) != cudaSuccess) return e;
    if ((e = mark(0)) != cudaSuccess) return e;
    if (sb.p.mesh.num_drawn == 0) {  // nothing to draw: the framebuffer stays as it is
        for (int k = 1; k < kStageEvents; ++k)
            if ((e = mark(k)) != cudaSuccess) return e;
        return cudaSuccess;
    }
    solo_vertex_kernel<S><<<blocks_for(sb.p.mesh.num_vertices), kBlock, 0, stream>>>(sb);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(1)) != cudaSuccess) return e;
    solo_face_kernel<<<blocks_for(sb.p.mesh.num_drawn), kBlock, 0, stream>>>(sb);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // stage events 2..4 (large, scan) have no kernel in this form
    for (int k = 2; k <= 4; ++k)
        if ((e = mark(k)) != cudaSuccess) return e;
    solo_bin_kernel<S><<<(unsigned)sb.bins.nbins, kBinThreads, 0, stream>>>(sb);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(5)) != cudaSuccess || (e = mark(6)) != cudaSuccess)
        return e;
    *launches += 3;
    return cudaSuccess;
}

template <int S>
cudaError_t launch_batch_binned_s(const BatchParams& bp, cudaStream_t stream, cudaEvent_t* ev, uint64_t* launches) {
    cudaError_t e;
    auto mark = [&](int k) { return ev ? cudaEventRecord(ev[k], stream) : cudaSuccess; };
    const size_t bin_bytes = sizeof(BinCounters) + sizeof(uint32_t) * (size_t)bp.bins.nbins;
    if ((e = cudaMemsetAsync(bp.counters, 0, kBatchCountersReset, stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bp.bins.counters, 0, bin_bytes, stream)) != cudaSuccess) return e;
    // phase events: 0 start, 1 after the (absent) clear kernel, 2 vertices, 3 faces, 4 after
    // the (absent) large-triangle phase, 5 bins
    if ((e = mark(0)) != cudaSuccess || (e = mark(1)) != cudaSuccess) return e;
    if (bp.vert_units) batch_bin_vertex_kernel<S><<<bp.vert_units, kBlock, 0, stream>>>(bp);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(2)) != cudaSuccess) return e;
    if (bp.face_units) batch_bin_face_kernel<<<bp.face_units, kBlock, 0, stream>>>(bp);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(3)) != cudaSuccess || (e = mark(4)) != cudaSuccess)
        return e;
    if (bp.tile_units) batch_bin_kernel<S><<<bp.tile_units, kBinThreads, 0, stream>>>(bp);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(5)) != cudaSuccess) return e;
    *launches += (bp.vert_units ? 1 : 0) + (bp.face_units ? 1 : 0) + (bp.tile_units ? 1 : 0);
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_draw_binned(const SoloBinned& sb, cudaStream_t stream, cudaEvent_t* stage_events,
                               uint64_t* launches) {
    switch (sb.p.u.shader) {
        case kFlat: return launch_solo_s<kFlat>(sb, stream, stage_events, launches);
        case kPhong: return launch_solo_s<kPhong>(sb, stream, stage_events, launches);
        case kPBR: return launch_solo_s<kPBR>(sb, stream, stage_events, launches);
        case kBlinnPhong: return launch_solo_s<kBlinnPhong>(sb, stream, stage_events, launches);
        case kGouraud: return launch_solo_s<kGouraud>(sb, stream, stage_events, launches);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch_binned(int shader, const BatchParams& bp, cudaStream_t stream, cudaEvent_t* phase_events,
                                uint64_t* launches) {
    switch (shader) {
        case kFlat: return launch_batch_binned_s<kFlat>(bp, stream, phase_events, launches);
        case kPhong: return launch_batch_binned_s<kPhong>(bp, stream, phase_events, launches);
        case kPBR: return launch_batch_binned_s<kPBR>(bp, stream, phase_events, launches);
        case kBlinnPhong: return launch_batch_binned_s<kBlinnPhong>(bp, stream, phase_events, launches);
        case kGouraud: return launch_batch_binned_s<kGouraud>(bp, stream, phase_events, launches);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace axr
