// Batched form: one persistent, cooperative launch renders many independent draws.
//
// The reference issues one drawMesh per mesh, each a full pass of its pipeline
// (src/tiled_pipeline.cpp:143-322). Here every draw of a batch has its own framebuffer,
// so the draws share nothing but the GPU, and one launch walks four phases over the
// work units of all draws, separated by grid barriers:
//   1. vertices   256-vertex units of every draw: screen cache + vertex-shader outputs
//   2. faces      256-face units in draw order: clip, cull, setup, small-triangle raster;
//                 large triangles go to one shared list with one item per 16x16 tile
//   3. large      warps take items of the shared list (4 per atomic), any draw
//   4. tiles      64-tile units, 8 tiles per warp: a warp reads a 16x16 tile's depth keys,
//                 shades the winners (compacted across the warp through shared memory),
//                 and writes the whole tile once. A draw that asks for a clear gets it
//                 fused here: the tile is staged in shared memory with the clear colour
//                 and depth, the winners are merged into it, and the 16x16 colour and
//                 depth boxes go out with two TMA tensor stores
//                 (cp.async.bulk.tensor, clipped at the framebuffer edge by the hardware),
//                 so every pixel of the frame is written exactly once.
// Units are handed out round-robin (unit u to CTA u mod grid); a table built by the host
// names each unit's draw, and the CTA stages that draw's DrawParams in shared memory
// (double-buffered, one __syncthreads per unit).
// Results are those of the per-draw path: the same device functions compute every
// value (draw_body.cuh), and the visibility keys give the same winners.
#include <cuda_runtime.h>

#include "batch.h"
#include "draw_body.cuh"

namespace axr {
namespace {

constexpr int kBatchBlock = 256;
constexpr int kBatchWarps = kBatchBlock / 32;
constexpr int kBatchMinBlocks = 3;  // 256 threads x 3 CTAs: at most 85 registers
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;

static_assert(sizeof(DrawParams) % 16 == 0, "DrawParams is copied as 16-byte words");
static_assert(offsetof(BatchDraw, p) % 16 == 0, "DrawParams is copied as 16-byte words");

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier of the cooperative launch (all CTAs are co-resident). The wait is
// bounded: after kBarrierTimeoutNs it sets kErrBarrier and the CTA leaves the kernel.
// With phase timing on, the last CTA to arrive at barrier k records the time.
__device__ bool grid_barrier(DevCounters* c, BatchProfile* prof, int k) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const uint32_t gen = ld_acquire(&c->bar_gen);
        __threadfence();
        if (atomicAdd(&c->bar_count, 1u) == gridDim.x - 1) {
            if (prof) prof->barrier_ns[k] = global_ns();
            atomicExch(&c->bar_count, 0u);
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (ld_acquire(&c->bar_gen) == gen) {
                if (global_ns() - t0 > kBarrierTimeoutNs) {
                    atomicOr(&c->error, kErrBarrier);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Phase timing at kernel exit: the last CTA out adds the four phase durations of this
// launch to the accumulators.
__device__ void profile_exit(BatchProfile* prof) {
    __syncthreads();
    if (threadIdx.x != 0) return;
    __threadfence();
    if (atomicAdd(&prof->exits, 1ull) != gridDim.x - 1) return;
    __threadfence();
    const unsigned long long end = global_ns();
    const volatile unsigned long long* b = prof->barrier_ns;
    const unsigned long long t0 = *reinterpret_cast<volatile unsigned long long*>(&prof->start);
    const unsigned long long t[5] = {t0, b[0], b[1], b[2], end};
    for (int k = 0; k < 4; ++k) atomicAdd(&prof->phase_ns[k], t[k + 1] > t[k] ? t[k + 1] - t[k] : 0ull);
    atomicAdd(&prof->launches, 1ull);
    prof->exits = 0ull;
}

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

// ---- TMA tensor store of a staged 16x16 tile (PTX ISA: cp.async.bulk.tensor, bulk_group)
__device__ __forceinline__ void tma_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tma_store_tile(const TensorMap128* map, const uint32_t* smem, int x, int y) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
                 :
                 : "l"(reinterpret_cast<uint64_t>(map)), "r"(s), "r"(x), "r"(y)
                 : "memory");
}

__device__ __forceinline__ void tma_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Wait until at most one committed group is still reading shared memory.
__device__ __forceinline__ void tma_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }

__device__ __forceinline__ void tma_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// One 16x16 tile of draw `p` (`dirty`: its flag was set): read its keys, shade the winners,
// write the tile. The caller skips tiles that are neither dirty nor to be cleared.
// stage: this warp's staging buffer (colour plane [256] then depth plane [256]);
// list: this warp's 256-entry pixel list. Returns whether a TMA store was committed.
template <int S>
__device__ bool tile_pass(const DrawParams& p, const UnitInfo& ui, const BatchDraw* bd, uint32_t tile, bool dirty,
                          uint32_t* stage, uint8_t* list, DevCounters* counters, bool stats) {
    const DevTarget& t = p.target;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const bool clear_c = (ui.flags & kBatchClearColor) != 0u, clear_d = (ui.flags & kBatchClearDepth) != 0u;
    const bool full = clear_c && clear_d;  // every pixel of the tile is rewritten
    const int tx = (int)(tile % (uint32_t)t.tiles_x), ty = (int)(tile / (uint32_t)t.tiles_x);
    const int lx = lane & 15, ly0 = lane >> 4;
    const int px = tx * kTile + lx;
    uint32_t* s_col = stage;
    float* s_dep = reinterpret_cast<float*>(stage + 256);
    const float cd = ui.clear_depth;
    const uint32_t cc = ui.clear_bgra;

    unsigned long long keys[8];
    unsigned ms[8];
    uint32_t nwin = 0;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int py = ty * kTile + ly0 + 2 * r;
        const bool in = px < t.width && py < t.height;
        keys[r] = (dirty && in) ? t.key[(uint32_t)py * (uint32_t)t.width + (uint32_t)px] : kEmptyKey;
        if (full) {
            s_col[(ly0 + 2 * r) * kTile + lx] = cc;
            s_dep[(ly0 + 2 * r) * kTile + lx] = cd;
        }
    }
    __syncwarp();
    // unclipped winners: pixel index into the list, tag parked in the colour staging slot
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const bool has = keys[r] != kEmptyKey;
        const bool win = has && (((uint32_t)keys[r]) & 8u) == 0u;
        ms[r] = __ballot_sync(0xFFFFFFFFu, win);
        if (win) {
            const int pix = (ly0 + 2 * r) * kTile + lx;
            list[nwin + (uint32_t)__popc(ms[r] & below)] = (uint8_t)pix;
            s_col[pix] = (uint32_t)keys[r];
        }
        nwin += (uint32_t)__popc(ms[r]);
    }
    __syncwarp();
    for (uint32_t base = 0; base < nwin; base += 32) {
        const uint32_t q = base + (uint32_t)lane;
        uint32_t pix = 0, bgra = cc;
        float z = cd;
        bool ok = false;
        if (q < nwin) {
            pix = list[q];
            const uint32_t tag = s_col[pix];
            const int gx = tx * kTile + (int)(pix & 15u), gy = ty * kTile + (int)(pix >> 4);
            const size_t idx = (size_t)gy * (size_t)t.width + (size_t)gx;
            const float old = clear_d ? cd : t.depth[idx];
            Screen s;
            VSOut vo[3];
            const uint32_t material = winner_inputs<S, true>(p, tag, s, vo);
            ok = shade_pixel<S>(p, gx, gy, material, s, vo, old, bgra, z);
            if (!full) {
                if (ok) {
                    t.color[idx] = bgra;
                    t.depth[idx] = z;
                } else {
                    if (clear_c) t.color[idx] = cc;
                    if (clear_d) t.depth[idx] = cd;
                }
            }
        }
        __syncwarp();  // every tag of this round is read before any slot is overwritten
        if (q < nwin && full) {
            s_col[pix] = ok ? bgra : cc;
            s_dep[pix] = ok ? z : cd;
        }
    }
    // clipped winners (rare): each lane re-clips its own pixels
#pragma unroll 1
    for (int r = 0; r < 8; ++r) {
        if (keys[r] == kEmptyKey || (((uint32_t)keys[r]) & 8u) == 0u) continue;
        const int gy = ty * kTile + ly0 + 2 * r;
        const int pix = (ly0 + 2 * r) * kTile + lx;
        const size_t idx = (size_t)gy * (size_t)t.width + (size_t)px;
        Screen s;
        VSOut vo[3];
        uint32_t material, bgra = cc;
        float z = cd;
        const float old = clear_d ? cd : t.depth[idx];
        const bool ok = clipped_inputs<S>(p, (uint32_t)keys[r], s, vo, material) &&
                        shade_pixel<S>(p, px, gy, material, s, vo, old, bgra, z);
        if (full) {
            s_col[pix] = ok ? bgra : cc;
            s_dep[pix] = ok ? z : cd;
        } else if (ok) {
            t.color[idx] = bgra;
            t.depth[idx] = z;
        } else {
            if (clear_c) t.color[idx] = cc;
            if (clear_d) t.depth[idx] = cd;
        }
    }
    // pixels without a key: the requested clear (a full clear is already staged)
    if (!full && (clear_c || clear_d)) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int py = ty * kTile + ly0 + 2 * r;
            if (keys[r] != kEmptyKey || px >= t.width || py >= t.height) continue;
            const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
            if (clear_c) t.color[idx] = cc;
            if (clear_d) t.depth[idx] = cd;
        }
    }
    // reset the keys and the flag for the next draw into this framebuffer
    if (dirty) {
#pragma unroll
        for (int r = 0; r < 8; ++r)
            if (keys[r] != kEmptyKey)
                t.key[(uint32_t)(ty * kTile + ly0 + 2 * r) * (uint32_t)t.width + (uint32_t)px] = kEmptyKey;
        if (lane == 0) {
            t.tile_flag[tile] = 0u;
            if (stats) atomicAdd(&counters->stat_tiles, 1ull);
        }
    }
    if (!full) return false;
    __syncwarp();
    if (ui.flags & kBatchTma) {
        tma_fence_smem();  // this lane's shared-memory writes -> visible to the TMA unit
        __syncwarp();
        if (lane == 0) {
            tma_store_tile(&bd->color_map, s_col, tx * kTile, ty * kTile);
            tma_store_tile(&bd->depth_map, reinterpret_cast<const uint32_t*>(s_dep), tx * kTile, ty * kTile);
            tma_commit();
        }
        return true;
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int py = ty * kTile + ly0 + 2 * r;
        if (px >= t.width || py >= t.height) continue;
        const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
        t.color[idx] = s_col[(ly0 + 2 * r) * kTile + lx];
        t.depth[idx] = s_dep[(ly0 + 2 * r) * kTile + lx];
    }
    return false;
}

template <int S>
__global__ void __launch_bounds__(kBatchBlock, kBatchMinBlocks) batch_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p[2];
    __shared__ UnitInfo s_u[2];
    __shared__ __align__(128) uint32_t s_stage[kBatchWarps][2][512];  // warp, buffer, colour|depth
    __shared__ uint8_t s_list[kBatchWarps][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool stats = bp.collect_stats != 0;

    BatchProfile* prof = bp.prof;
    if (prof && blockIdx.x == 0 && threadIdx.x == 0) prof->start = global_ns();
    const uint32_t face_base = bp.vert_units, tile_base = bp.vert_units + bp.face_units;

    // ---- phase 1: vertices
    int buf = 0;
    for (uint32_t u = blockIdx.x; u < bp.vert_units; u += gridDim.x, buf ^= 1) {
        stage_unit(bp, u, &s_p[buf], &s_u[buf]);
        __syncthreads();
        const DrawParams& p = s_p[buf];
        const uint32_t i = s_u[buf].local * kVertUnit + threadIdx.x;
        if (i < p.mesh.num_vertices) vertex_one<S>(p, i);
    }
    if (!grid_barrier(bp.counters, prof, 0)) return;

    // ---- phase 2: faces
    for (uint32_t u = blockIdx.x; u < bp.face_units; u += gridDim.x, buf ^= 1) {
        stage_unit(bp, face_base + u, &s_p[buf], &s_u[buf]);
        __syncthreads();
        const DrawParams& p = s_p[buf];
        GeomStats st = {0, 0, 0};
        uint32_t single_tile = kNoTile;
        const uint32_t o = s_u[buf].local * kFaceUnit + threadIdx.x;
        if (o < p.mesh.num_drawn) geometry_one<true>(p, o, st, single_tile);
        geometry_warp_tail(p.target, bp.counters, stats, st, single_tile);
    }
    if (!grid_barrier(bp.counters, prof, 1)) return;

    // ---- phase 3: large-triangle tiles of all draws
    {
        DevCounters* c = bp.counters;
        const uint32_t n_items = min(ld_acquire(&c->item_count), bp.item_cap);
        const uint32_t n_tris = min(ld_acquire(&c->large_count), bp.large_cap);
        uint32_t frags = 0;
        for (;;) {
            uint32_t first = 0;
            if (lane == 0) first = atomicAdd(&c->item_head, kItemsPerGrab);
            first = __shfl_sync(0xFFFFFFFFu, first, 0);
            if (first >= n_items) break;
            const uint32_t last = min(first + kItemsPerGrab, n_items);
            for (uint32_t it = first; it < last; ++it) {
                const LargeItem item = bp.items[it];
                if (item.tri >= n_tris) continue;  // reserved slot of a triangle rasterised elsewhere
                const DevTarget t = bp.draws[bp.large_draw[item.tri]].p.target;
                Edges e;
                uint32_t tag;
                load_large(&bp.large[item.tri], e, tag);
                large_tile(t, e, tag, item.tile, frags);
            }
        }
        if (stats) {
            const uint32_t f = __reduce_add_sync(0xFFFFFFFFu, frags);
            if (lane == 0 && f) atomicAdd(&c->stat_fragments, (unsigned long long)f);
        }
    }
    if (!grid_barrier(bp.counters, prof, 2)) return;

    // ---- phase 4: tiles (key scan, shading, fused clear, tile write-out); each warp takes
    // 8 consecutive tiles of the unit, their flags read with one load per lane
    int sbuf = 0;
    for (uint32_t u = blockIdx.x; u < bp.tile_units; u += gridDim.x, buf ^= 1) {
        stage_unit(bp, tile_base + u, &s_p[buf], &s_u[buf]);
        __syncthreads();
        const DrawParams& p = s_p[buf];
        const UnitInfo& ui = s_u[buf];
        const uint32_t ntiles = (uint32_t)p.target.tiles_x * (uint32_t)p.target.tiles_y;
        const uint32_t first = ui.local * kTileUnit + (uint32_t)warp * kTilesPerWarp;
        const bool clears = (ui.flags & (kBatchClearColor | kBatchClearDepth)) != 0u;
        const bool flag = lane < (int)kTilesPerWarp && first + (uint32_t)lane < ntiles &&
                          ld_volatile(&p.target.tile_flag[first + (uint32_t)lane]) != 0u;
        const unsigned dirty = __ballot_sync(0xFFFFFFFFu, flag);
        for (uint32_t j = 0; j < kTilesPerWarp; ++j) {
            const uint32_t tile = first + j;
            if (tile >= ntiles) break;
            const bool d = (dirty >> j) & 1u;
            if (!d && !clears) continue;
            // the store issued from this buffer two tiles ago must have read it
            if (lane == 0) tma_wait_read_1();
            __syncwarp();
            if (tile_pass<S>(p, ui, &bp.draws[ui.draw], tile, d, s_stage[warp][sbuf], s_list[warp], bp.counters,
                             stats))
                sbuf ^= 1;
        }
    }
    if (lane == 0) tma_wait_all();
    if (prof) profile_exit(prof);
}

template <int S>
cudaError_t launch_batch_s(const BatchParams& bp, int num_sms, cudaStream_t stream, uint64_t* launches) {
    // resident CTAs per SM of this instantiation, per device (a cooperative launch must not
    // exceed it)
    constexpr int kMaxDev = 64;
    static int blocks_per_sm[kMaxDev] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    if (blocks_per_sm[dev] == 0) {
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<S>, kBatchBlock, 0);
        if (e != cudaSuccess) return e;
        if (n < 1) return cudaErrorInvalidConfiguration;
        blocks_per_sm[dev] = n;
    }
    const unsigned grid = (unsigned)(blocks_per_sm[dev] * num_sms);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kBatchBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaMemsetAsync(bp.counters, 0, kBatchCountersReset, stream);
    if (e != cudaSuccess) return e;
    if (bp.prof && (e = cudaMemsetAsync(&bp.prof->exits, 0, sizeof(bp.prof->exits), stream)) != cudaSuccess) return e;
    e = cudaLaunchKernelEx(&cfg, batch_kernel<S>, bp);
    if (e == cudaSuccess) *launches += 1;
    return e;
}

}  // namespace

cudaError_t launch_batch(int shader, const BatchParams& bp, int num_sms, cudaStream_t stream, uint64_t* launches) {
    switch (shader) {
        case kFlat: return launch_batch_s<kFlat>(bp, num_sms, stream, launches);
        case kPhong: return launch_batch_s<kPhong>(bp, num_sms, stream, launches);
        case kPBR: return launch_batch_s<kPBR>(bp, num_sms, stream, launches);
        case kBlinnPhong: return launch_batch_s<kBlinnPhong>(bp, num_sms, stream, launches);
        case kGouraud: return launch_batch_s<kGouraud>(bp, num_sms, stream, launches);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace axr
