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
//   4. tiles      tile units, one warp per 16x16 tile: a warp reads the tile's depth keys,
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
#include "tma.cuh"
#include "unit.cuh"

namespace axr {
namespace {

constexpr int kBatchBlock = 256;
constexpr int kBatchWarps = kBatchBlock / 32;
constexpr int kBatchMinBlocks = 3;  // 256 threads x 3 CTAs: at most 85 registers
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;

// Resident 256-thread CTAs per SM the phased face kernel is compiled for (5: at most 51
// registers; its shared memory, 15 KB per CTA, allows more).
#ifndef AXR_FACE_MIN_BLOCKS
#define AXR_FACE_MIN_BLOCKS 5
#endif

// Resident 256-thread CTAs per SM the phased tile kernel is compiled for (4: at most 64
// registers; its shared memory, 36 KB per CTA, allows 6).
#ifndef AXR_TILE_MIN_BLOCKS
#define AXR_TILE_MIN_BLOCKS 4
#endif

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
// bounded: after timeout_ns (kBarrierTimeoutNs unless a caller passes less) it sets
// kErrBarrier and returns false, and the CTA leaves the kernel.
// With phase timing on, the last CTA to arrive at barrier k records the time.
__device__ bool grid_barrier(DevCounters* c, BatchProfile* prof, int k,
                             unsigned long long timeout_ns = kBarrierTimeoutNs) {
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
                if (global_ns() - t0 > timeout_ns) {
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

// ---- the tile pass, in three steps over one 16x16 tile of draw `p`:
//   tile_scan    (warp) keys -> pixel lists in shared memory: unclipped winners from the
//                front of `list`, clipped ones from the back, their tags parked in the
//                colour staging slots; keys and flag reset; pixels without a key get the
//                requested clear (staged when both planes are cleared, else written)
//   shade_winner (thread) one unclipped winner: fragment, merged into the staging slots
//                or written to the framebuffer
//   tile_finish  (warp) the clipped winners (rare), then the staged tile out with two
//                TMA tensor stores (or plain stores when the pitch has no tensor map)
// `stage` is the tile's staging buffer: colour plane [256] then depth plane [256].
struct TileCtx {
    uint32_t tile;
    int tx, ty;
    bool clear_c, clear_d, full;
};

__device__ __forceinline__ TileCtx tile_ctx(const DevTarget& t, const UnitInfo& ui, uint32_t tile) {
    TileCtx c;
    c.tile = tile;
    c.tx = (int)(tile % (uint32_t)t.tiles_x);
    c.ty = (int)(tile / (uint32_t)t.tiles_x);
    c.clear_c = (ui.flags & kBatchClearColor) != 0u;
    c.clear_d = (ui.flags & kBatchClearDepth) != 0u;
    c.full = c.clear_c && c.clear_d;
    return c;
}

// Returns nwin | nclip << 16 (lane-uniform).
__device__ uint32_t tile_scan(const DrawParams& p, const UnitInfo& ui, const TileCtx& c, bool dirty, uint32_t* stage,
                              uint8_t* list, DevCounters* counters, bool stats) {
    const DevTarget& t = p.target;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int lx = lane & 15, ly0 = lane >> 4;
    const int px = c.tx * kTile + lx;
    uint32_t* s_col = stage;
    float* s_dep = reinterpret_cast<float*>(stage + 256);
    const float cd = ui.clear_depth;
    const uint32_t cc = ui.clear_bgra;
    uint32_t nwin = 0, nclip = 0;
    // all eight keys first: the resets below would otherwise keep the compiler from
    // issuing a row's load before the previous row's store (one load in flight)
    unsigned long long keys[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int py = c.ty * kTile + ly0 + 2 * r;
        const bool in = px < t.width && py < t.height;
        keys[r] = (dirty && in) ? __ldcg(t.key + (size_t)py * (size_t)t.width + (size_t)px) : kEmptyKey;
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int ly = ly0 + 2 * r, py = c.ty * kTile + ly, pix = ly * kTile + lx;
        const bool in = px < t.width && py < t.height;
        const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
        const unsigned long long key = keys[r];
        const bool has = key != kEmptyKey;
        const bool clipped = has && (((uint32_t)key) & 8u) != 0u;
        const unsigned mw = __ballot_sync(0xFFFFFFFFu, has && !clipped);
        const unsigned mc = __ballot_sync(0xFFFFFFFFu, clipped);
        if (has) {
            t.key[idx] = kEmptyKey;  // reset for the next draw into this framebuffer
            s_col[pix] = (uint32_t)key;
            if (clipped)
                list[255u - (nclip + (uint32_t)__popc(mc & below))] = (uint8_t)pix;
            else
                list[nwin + (uint32_t)__popc(mw & below)] = (uint8_t)pix;
        } else if (c.full) {
            s_col[pix] = cc;
            s_dep[pix] = cd;
        } else if (in) {
            if (c.clear_c) t.color[idx] = cc;
            if (c.clear_d) t.depth[idx] = cd;
        }
        nwin += (uint32_t)__popc(mw);
        nclip += (uint32_t)__popc(mc);
    }
    if (dirty && lane == 0) {
        t.tile_flag[c.tile] = 0u;
        if (stats) {
            atomicAdd(&counters->stat_tiles, 1ull);
            atomicAdd(&counters->stat_shaded, (unsigned long long)(nwin + nclip));
        }
    }
    return nwin | (nclip << 16);
}

// Merge one shaded (or rejected) fragment of pixel `pix` of the tile.
__device__ __forceinline__ void tile_put(const DevTarget& t, const UnitInfo& ui, const TileCtx& c, uint32_t* stage,
                                         uint32_t pix, size_t idx, bool ok, uint32_t bgra, float z) {
    if (c.full) {
        stage[pix] = ok ? bgra : ui.clear_bgra;
        reinterpret_cast<float*>(stage + 256)[pix] = ok ? z : ui.clear_depth;
    } else if (ok) {
        t.color[idx] = bgra;
        t.depth[idx] = z;
    } else {
        if (c.clear_c) t.color[idx] = ui.clear_bgra;
        if (c.clear_d) t.depth[idx] = ui.clear_depth;
    }
}

template <int S>
__device__ __forceinline__ void shade_winner(const DrawParams& p, const UnitInfo& ui, const TileCtx& c, uint32_t* stage,
                                             uint32_t pix) {
    const DevTarget& t = p.target;
    const uint32_t tag = stage[pix];
    const int gx = c.tx * kTile + (int)(pix & 15u), gy = c.ty * kTile + (int)(pix >> 4);
    const size_t idx = (size_t)gy * (size_t)t.width + (size_t)gx;
    const float old = c.clear_d ? ui.clear_depth : t.depth[idx];
    uint32_t bgra = 0u;
    float z = 0.0f;
    const bool ok = shade_unclipped<S, true>(p, tag, gx, gy, old, bgra, z);
    tile_put(t, ui, c, stage, pix, idx, ok, bgra, z);
}

// Returns whether a TMA store was committed.
template <int S>
__device__ bool tile_finish(const DrawParams& p, const UnitInfo& ui, const BatchDraw* bd, const TileCtx& c,
                            uint32_t* stage, const uint8_t* list, uint32_t nclip) {
    const DevTarget& t = p.target;
    const int lane = threadIdx.x & 31;
#pragma unroll 1
    for (uint32_t q = (uint32_t)lane; q < nclip; q += 32) {
        const uint32_t pix = list[255u - q];
        const uint32_t tag = stage[pix];
        const int gx = c.tx * kTile + (int)(pix & 15u), gy = c.ty * kTile + (int)(pix >> 4);
        const size_t idx = (size_t)gy * (size_t)t.width + (size_t)gx;
        const float old = c.clear_d ? ui.clear_depth : t.depth[idx];
        uint32_t bgra = 0u;
        float z = 0.0f;
        const bool ok = shade_clipped_px<S>(p, tag, gx, gy, old, &bgra, &z);
        tile_put(t, ui, c, stage, pix, idx, ok, bgra, z);
    }
    if (!c.full) return false;
    __syncwarp();
    if (ui.flags & kBatchTma) {
        tma_fence_smem();  // this lane's shared-memory writes -> visible to the TMA unit
        __syncwarp();
        if (lane == 0) {
            tma_store_tile(&bd->color_map, stage, c.tx * kTile, c.ty * kTile);
            tma_store_tile(&bd->depth_map, stage + 256, c.tx * kTile, c.ty * kTile);
            tma_commit();
        }
        return true;
    }
    const int lx = lane & 15, ly0 = lane >> 4, px = c.tx * kTile + lx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int py = c.ty * kTile + ly0 + 2 * r;
        if (px >= t.width || py >= t.height) continue;
        const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
        t.color[idx] = stage[(ly0 + 2 * r) * kTile + lx];
        t.depth[idx] = reinterpret_cast<const float*>(stage + 256)[(ly0 + 2 * r) * kTile + lx];
    }
    return false;
}

// The whole tile pass by one warp (persistent form). Returns whether a TMA store was committed.
template <int S>
__device__ bool tile_pass(const DrawParams& p, const UnitInfo& ui, const BatchDraw* bd, uint32_t tile, bool dirty,
                          uint32_t* stage, uint8_t* list, DevCounters* counters, bool stats) {
    const TileCtx c = tile_ctx(p.target, ui, tile);
    const uint32_t n = tile_scan(p, ui, c, dirty, stage, list, counters, stats);
    const uint32_t nwin = n & 0xFFFFu, nclip = n >> 16;
    __syncwarp();
#pragma unroll 1
    for (uint32_t q = threadIdx.x & 31u; q < nwin; q += 32) shade_winner<S>(p, ui, c, stage, list[q]);
    __syncwarp();
    return tile_finish<S>(p, ui, bd, c, stage, list, nclip);
}

// ---- phase bodies, shared by the persistent and the phased forms
template <int S>
__device__ __forceinline__ void vertex_unit(const DrawParams& p, const UnitInfo& ui) {
    const uint32_t i = ui.local * kVertUnit + threadIdx.x;
    if (i < p.mesh.num_vertices) vertex_one<S>(p, i);
}

// kCoherent: the vertex cache was written earlier in the same launch
template <bool kCoherent>
__device__ __forceinline__ void face_unit(const DrawParams& p, const UnitInfo& ui, DevCounters* c, bool stats) {
    GeomStats st = {0, 0, 0, 0};
    uint32_t single_tile = kNoTile;
    const uint32_t o = ui.local * kFaceUnit + threadIdx.x;
    if (o < p.mesh.num_drawn) geometry_one<kCoherent>(p, o, st, single_tile);
    geometry_warp_tail(p.target, c, stats, st, single_tile);
}

// Large-triangle tile items of all draws, strided over every warp of the grid (items are
// alike, 256 pixels each, so a static split balances without a shared counter).
__device__ __forceinline__ void large_items(const BatchParams& bp, bool stats) {
    const int lane = threadIdx.x & 31;
    DevCounters* c = bp.counters;
    const uint32_t n_items = min(ld_acquire(&c->item_count), bp.item_cap);
    const uint32_t n_tris = min(ld_acquire(&c->large_count), bp.large_cap);
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    uint32_t frags = 0, tested = 0;
    for (uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < n_items; it += warps) {
        const LargeItem item = bp.items[it];
        if (item.tri >= n_tris) continue;  // reserved slot of a triangle rasterised elsewhere
        const DevTarget t = bp.draws[bp.large_draw[item.tri]].p.target;
        Edges e;
        uint32_t tag;
        load_large(&bp.large[item.tri], e, tag);
        large_tile(t, e, tag, item.tile, frags, tested);
    }
    if (stats) {
        const uint32_t f = __reduce_add_sync(0xFFFFFFFFu, frags);
        const uint32_t te = __reduce_add_sync(0xFFFFFFFFu, tested);
        if (lane == 0 && f) atomicAdd(&c->stat_fragments, (unsigned long long)f);
        if (lane == 0 && te) atomicAdd(&c->stat_tested, (unsigned long long)te);
    }
}

// Both planes of a tile without keys set to the clear values with direct stores: 8 pixels
// of one row per lane (two 16-byte stores per plane) when the tile lies inside a
// framebuffer whose width is a multiple of 4, one pixel per store otherwise.
__device__ __forceinline__ void clear_tile(const DevTarget& t, uint32_t tile, uint32_t cc, float cd) {
    const int lane = threadIdx.x & 31;
    const int tx = (int)(tile % (uint32_t)t.tiles_x), ty = (int)(tile / (uint32_t)t.tiles_x);
    const int x0 = tx * kTile, y0 = ty * kTile;
    if ((t.width & 3) == 0 && x0 + kTile <= t.width && y0 + kTile <= t.height) {
        const int py = y0 + (lane >> 1), px = x0 + 8 * (lane & 1);
        const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
        const uint4 c4 = make_uint4(cc, cc, cc, cc);
        const float4 d4 = make_float4(cd, cd, cd, cd);
        uint4* c = reinterpret_cast<uint4*>(t.color + idx);
        float4* d = reinterpret_cast<float4*>(t.depth + idx);
        c[0] = c4;
        c[1] = c4;
        d[0] = d4;
        d[1] = d4;
        return;
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int px = x0 + (lane & 15), py = y0 + (lane >> 4) + 2 * r;
        if (px >= t.width || py >= t.height) continue;
        const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
        t.color[idx] = cc;
        t.depth[idx] = cd;
    }
}

// A warp's tiles of a tile unit: their flags with one load per lane, then tile_pass on each
// tile that is dirty or to be cleared. *sbuf alternates the warp's two staging buffers.
template <int S>
__device__ __forceinline__ void tile_unit(const BatchParams& bp, const DrawParams& p, const UnitInfo& ui,
                                          uint32_t* stage2, uint8_t* list, int* sbuf, bool stats) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tpw = bp.tiles_per_warp;
    const uint32_t ntiles = (uint32_t)p.target.tiles_x * (uint32_t)p.target.tiles_y;
    const uint32_t first = (ui.local * kUnitWarps + (uint32_t)warp) * tpw;
    const bool clears = (ui.flags & (kBatchClearColor | kBatchClearDepth)) != 0u;
    const bool flag = (uint32_t)lane < tpw && first + (uint32_t)lane < ntiles &&
                      ld_volatile(&p.target.tile_flag[first + (uint32_t)lane]) != 0u;
    const unsigned dirty = __ballot_sync(0xFFFFFFFFu, flag);
    const bool full_clear = (ui.flags & (kBatchClearColor | kBatchClearDepth)) == (kBatchClearColor | kBatchClearDepth);
    for (uint32_t j = 0; j < tpw; ++j) {
        const uint32_t tile = first + j;
        if (tile >= ntiles) break;
        const bool d = (dirty >> j) & 1u;
        if (!d && !clears) continue;
        if (!d && full_clear) {
            clear_tile(p.target, tile, ui.clear_bgra, ui.clear_depth);
            continue;
        }
        // the store issued from this buffer two tiles ago must have read it
        if (lane == 0) tma_wait_read_1();
        __syncwarp();
        if (tile_pass<S>(p, ui, &bp.draws[ui.draw], tile, d, stage2 + 512 * *sbuf, list, bp.counters, stats))
            *sbuf ^= 1;
    }
}

// ---- persistent form: one cooperative launch, phases behind grid barriers
template <int S>
__global__ void __launch_bounds__(kBatchBlock, kBatchMinBlocks) batch_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p[2];
    __shared__ UnitInfo s_u[2];
    __shared__ __align__(128) uint32_t s_stage[kBatchWarps][2 * 512];  // warp: 2 x (colour | depth)
    __shared__ uint8_t s_list[kBatchWarps][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool stats = bp.collect_stats != 0;
    BatchProfile* prof = bp.prof;
    if (prof && blockIdx.x == 0 && threadIdx.x == 0) prof->start = global_ns();
    const uint32_t face_base = bp.vert_units, tile_base = bp.vert_units + bp.face_units;
    int buf = 0;
    for (uint32_t u = blockIdx.x; u < bp.vert_units; u += gridDim.x, buf ^= 1) {
        stage_unit(bp, u, &s_p[buf], &s_u[buf]);
        __syncthreads();
        vertex_unit<S>(s_p[buf], s_u[buf]);
    }
    if (!grid_barrier(bp.counters, prof, 0)) return;
    for (uint32_t u = blockIdx.x; u < bp.face_units; u += gridDim.x, buf ^= 1) {
        stage_unit(bp, face_base + u, &s_p[buf], &s_u[buf]);
        __syncthreads();
        face_unit<true>(s_p[buf], s_u[buf], bp.counters, stats);
    }
    if (!grid_barrier(bp.counters, prof, 1)) return;
    large_items(bp, stats);
    if (!grid_barrier(bp.counters, prof, 2)) return;
    int sbuf = 0;
    for (uint32_t u = blockIdx.x; u < bp.tile_units; u += gridDim.x, buf ^= 1) {
        stage_unit(bp, tile_base + u, &s_p[buf], &s_u[buf]);
        __syncthreads();
        tile_unit<S>(bp, s_p[buf], s_u[buf], s_stage[warp], s_list[warp], &sbuf, stats);
    }
    if (lane == 0) tma_wait_all();
    if (prof) profile_exit(prof);
}

// ---- phased form: one launch per phase, one CTA per work unit (large: persistent warps)
template <int S>
__global__ void __launch_bounds__(kBatchBlock) batch_vertex_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p;
    __shared__ UnitInfo s_u;
    stage_unit(bp, blockIdx.x, &s_p, &s_u);
    __syncthreads();
    vertex_unit<S>(s_p, s_u);
}

__global__ void __launch_bounds__(kBatchBlock, AXR_FACE_MIN_BLOCKS) batch_face_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p;
    __shared__ UnitInfo s_u;
    __shared__ FaceJob s_jobs[kBatchBlock];
    __shared__ uint32_t s_count;
    if (threadIdx.x == 0) s_count = 0u;
    stage_unit(bp, bp.vert_units + blockIdx.x, &s_p, &s_u);
    __syncthreads();
    geometry_compacted(s_p, s_u.local * kFaceUnit + threadIdx.x, bp.counters, bp.collect_stats != 0, s_jobs,
                       &s_count);
}

__global__ void __launch_bounds__(kBatchBlock) batch_large_kernel(const __grid_constant__ BatchParams bp) {
    large_items(bp, bp.collect_stats != 0);
}

// Tile pass of the phased form: one CTA per unit of 8 x tiles_per_warp consecutive tiles
// (at most 32). Warp 0 reads the unit's tile flags with one load per lane. Tiles without
// keys whose two planes are to be cleared are cleared directly by the warps (no staging,
// no barrier). The other tiles go through the staged pass in rounds of eight, one per
// warp: each warp scans its tile, then all 256 threads shade the round's winners together
// (balanced across the eight tiles), then each warp finishes its tile. A warp's two
// staging buffers alternate after each committed TMA store, so a tile's store overlaps
// the next round.
template <int S>
__global__ void __launch_bounds__(kBatchBlock, AXR_TILE_MIN_BLOCKS) batch_tile_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ __align__(16) DrawParams s_p;
    __shared__ UnitInfo s_u;
    __shared__ __align__(128) uint32_t s_stage[kBatchWarps][2][512];
    __shared__ uint8_t s_list[kBatchWarps][256];
    __shared__ uint32_t s_n[kBatchWarps], s_buf[kBatchWarps], s_tile[kBatchWarps];
    __shared__ uint32_t s_dirty;
    __shared__ __align__(128) uint32_t s_clear[2][256];  // a cleared tile: colour, depth (TMA source)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool stats = bp.collect_stats != 0;
    stage_unit(bp, bp.vert_units + bp.face_units + blockIdx.x, &s_p, &s_u);
    __syncthreads();
    const DrawParams& p = s_p;
    const UnitInfo& ui = s_u;
    // a fully cleared draw with tensor maps: its key-less tiles go out as TMA stores of one
    // cleared tile in shared memory (no clear kernel; every pixel of the frame written once)
    const bool tma_clear = (ui.flags & (kBatchClearColor | kBatchClearDepth)) == (kBatchClearColor | kBatchClearDepth) &&
                           (ui.flags & kBatchTma) && !(ui.flags & kBatchClearedApart);
    if (tma_clear) {
        s_clear[0][threadIdx.x] = ui.clear_bgra;
        s_clear[1][threadIdx.x] = __float_as_uint(ui.clear_depth);
        tma_fence_smem();  // visible to the TMA unit after the barrier below
    }
    const uint32_t ntiles = (uint32_t)p.target.tiles_x * (uint32_t)p.target.tiles_y;
    const uint32_t unit = kUnitWarps * bp.tiles_per_warp;  // <= 32
    const uint32_t first = ui.local * unit;
    const uint32_t count = min(unit, ntiles - first);
    if (warp == 0) {
        const bool f = (uint32_t)lane < count && ld_volatile(&p.target.tile_flag[first + (uint32_t)lane]) != 0u;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, f);
        if (lane == 0) s_dirty = m;
    }
    __syncthreads();
    const unsigned all = count >= 32u ? 0xFFFFFFFFu : ((1u << count) - 1u);
    const unsigned dirty = s_dirty;
    const bool clears = (ui.flags & (kBatchClearColor | kBatchClearDepth)) != 0u;
    const bool full = (ui.flags & (kBatchClearColor | kBatchClearDepth)) == (kBatchClearColor | kBatchClearDepth);
    // key-less tiles with a full clear, spread over the warps (unless the clear kernel has
    // written them already): TMA stores of the cleared tile, issued by the warp's lane 0 and
    // read back from shared memory before the CTA exits (one issuing thread per tile
    // measured 1% slower); direct stores without tensor maps
    if (full && !(ui.flags & kBatchClearedApart)) {
        unsigned clean = all & ~dirty;
        const BatchDraw* bd = &bp.draws[ui.draw];
        for (int k = 0; clean; ++k) {
            const int t = __ffs(clean) - 1;
            clean &= clean - 1u;
            if ((k & (kBatchWarps - 1)) != warp) continue;
            const uint32_t tile = first + (uint32_t)t;
            if (tma_clear) {
                if (lane == 0) {
                    const int x = (int)(tile % (uint32_t)p.target.tiles_x) * kTile;
                    const int y = (int)(tile / (uint32_t)p.target.tiles_x) * kTile;
                    tma_store_tile(&bd->color_map, s_clear[0], x, y);
                    tma_store_tile(&bd->depth_map, s_clear[1], x, y);
                    tma_commit();
                }
            } else {
                clear_tile(p.target, tile, ui.clear_bgra, ui.clear_depth);
            }
        }
    }
    // staged tiles: the dirty ones, plus the key-less ones when only one plane is cleared
    unsigned work = full ? dirty : (clears ? all : dirty);
    uint32_t sbuf = 0;  // the buffer this warp stages into; never the newest committed store's
    while (work) {
        // this round: the next eight tiles of `work`, the w-th to warp w
        int mine = -1;
#pragma unroll
        for (int w = 0; w < kBatchWarps; ++w) {
            if (!work) break;
            const int t = __ffs(work) - 1;
            work &= work - 1u;
            if (w == warp) mine = t;
        }
        const uint32_t tile = first + (uint32_t)(mine < 0 ? 0 : mine);
        uint32_t* stage = s_stage[warp][sbuf];
        const TileCtx c = tile_ctx(p.target, ui, tile);
        uint32_t n = 0;
        if (mine >= 0) {
            if (lane == 0) tma_wait_read_1();  // an older store from this buffer has read it
            __syncwarp();
            n = tile_scan(p, ui, c, (dirty >> mine) & 1u, stage, s_list[warp], bp.counters, stats);
        }
        if (lane == 0) {
            s_n[warp] = n & 0xFFFFu;
            s_buf[warp] = sbuf;
            s_tile[warp] = tile;
        }
        __syncthreads();
        uint32_t pre[kBatchWarps + 1];
        pre[0] = 0;
#pragma unroll
        for (int w = 0; w < kBatchWarps; ++w) pre[w + 1] = pre[w] + s_n[w];
        for (uint32_t q = threadIdx.x; q < pre[kBatchWarps]; q += kBatchBlock) {
            int w = 0;
#pragma unroll
            for (int k = 1; k < kBatchWarps; ++k) w += q >= pre[k] ? 1 : 0;
            shade_winner<S>(p, ui, tile_ctx(p.target, ui, s_tile[w]), s_stage[w][s_buf[w]], s_list[w][q - pre[w]]);
        }
        __syncthreads();
        if (mine >= 0 && tile_finish<S>(p, ui, &bp.draws[ui.draw], c, stage, s_list[warp], n >> 16)) sbuf ^= 1u;
        __syncthreads();  // s_list, s_n, s_buf and s_tile are rewritten by the next round
    }
    // the staging buffers and the cleared tile must have been read before the CTA exits
    // (a thread that committed no store group passes at once)
    tma_wait_read_0();
}

// Clear of both planes of the phased form's fully cleared draws, in spans of kClearUnit
// pixels of one draw with 16-byte stores (planes are 256-byte aligned and spans start at
// multiples of 4 pixels). One CTA per SM walks the spans: 16-byte stores from 256 threads
// per SM reach the HBM write rate.
__global__ void __launch_bounds__(kBatchBlock) batch_clear_kernel(const __grid_constant__ BatchParams bp) {
    const uint2* units = reinterpret_cast<const uint2*>(bp.units) + bp.vert_units + bp.face_units + bp.tile_units;
    for (uint32_t u = blockIdx.x; u < bp.clear_units; u += gridDim.x) {
        const uint2 r = __ldg(units + u);
        const BatchDraw* bd = &bp.draws[r.x];
        uint32_t* color = bd->p.target.color;
        float* depth = bd->p.target.depth;
        const size_t n = (size_t)bd->p.target.width * (size_t)bd->p.target.height;
        const uint32_t cc = __ldg(&bd->clear_bgra);
        const float cd = __ldg(&bd->clear_depth);
        const size_t lo = (size_t)r.y * kClearUnit, hi = min(n, lo + kClearUnit);
        const uint4 c4 = make_uint4(cc, cc, cc, cc);
        const float4 d4 = make_float4(cd, cd, cd, cd);
        const size_t v_hi = lo + ((hi - lo) & ~size_t(3));
        for (size_t i = lo + 4 * (size_t)threadIdx.x; i < v_hi; i += 4 * (size_t)kBatchBlock) {
            *reinterpret_cast<uint4*>(color + i) = c4;
            *reinterpret_cast<float4*>(depth + i) = d4;
        }
        for (size_t i = v_hi + threadIdx.x; i < hi; i += kBatchBlock) {
            color[i] = cc;
            depth[i] = cd;
        }
    }
}

__global__ void merge_counters_kernel(DevCounters* dst, DevCounters* src) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const uint32_t err = src->error;
    if (err) atomicOr(&dst->error, err);
    src->error = 0u;
    unsigned long long* d = &dst->stat_triangles;
    unsigned long long* s = &src->stat_triangles;
    for (int k = 0; k < 6; ++k) {  // stat_triangles .. stat_shaded
        if (s[k]) atomicAdd(&d[k], s[k]);
        s[k] = 0ull;
    }
}

// Failure-path probe: CTA 0 waits at a grid barrier that CTA 1 never reaches, so the
// bounded wait gives up after timeout_ns and sets kErrBarrier.
__global__ void barrier_probe_kernel(DevCounters* c, unsigned long long timeout_ns) {
    if (blockIdx.x != 0) return;
    grid_barrier(c, nullptr, 0, timeout_ns);
}

template <int S>
cudaError_t launch_batch_s(const BatchParams& bp, int form, int num_sms, cudaStream_t stream, cudaEvent_t* ev,
                           uint64_t* launches, bool clear_late) {
    cudaError_t e = cudaMemsetAsync(bp.counters, 0, kBatchCountersReset, stream);
    if (e != cudaSuccess) return e;
    if (form == kFormPhased) {
        auto mark = [&](int k) { return ev ? cudaEventRecord(ev[k], stream) : cudaSuccess; };
        // at the HBM write rate; running it beside the vertex and face phases of the same
        // draws (a side stream) measured no faster, since their key atomics then wait on its
        // writes. The raster phases touch only keys and tile flags, so the clear may also
        // run just before the tile pass (clear_late).
        auto clear = [&]() -> cudaError_t {
            if (!bp.clear_units) return cudaSuccess;
            const unsigned g = min(bp.clear_units, (unsigned)num_sms);
            batch_clear_kernel<<<g, kBatchBlock, 0, stream>>>(bp);
            *launches += 1;
            return cudaGetLastError();
        };
        if ((e = mark(0)) != cudaSuccess) return e;
        if (!clear_late && (e = clear()) != cudaSuccess) return e;
        if ((e = mark(1)) != cudaSuccess) return e;
        if (bp.vert_units) batch_vertex_kernel<S><<<bp.vert_units, kBatchBlock, 0, stream>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(2)) != cudaSuccess) return e;
        if (bp.face_units) batch_face_kernel<<<bp.face_units, kBatchBlock, 0, stream>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(3)) != cudaSuccess) return e;
        // 16 CTAs per SM, about three waves of the 5 resident: the items are strided over
        // all warps of the grid, and the later waves even out the first waves' tails (5 per SM
        // measured 3.041 ms per 512-draw step, 8: 3.027, 10: 3.022, 16: 3.018, 32: 3.020)
        if (bp.face_units) batch_large_kernel<<<(unsigned)num_sms * 16u, kBatchBlock, 0, stream>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (clear_late && (e = clear()) != cudaSuccess) return e;
        if ((e = mark(4)) != cudaSuccess) return e;
        if (bp.tile_units) batch_tile_kernel<S><<<bp.tile_units, kBatchBlock, 0, stream>>>(bp);
        if ((e = cudaGetLastError()) != cudaSuccess || (e = mark(5)) != cudaSuccess) return e;
        *launches += (bp.vert_units ? 1 : 0) + (bp.face_units ? 2 : 0) + (bp.tile_units ? 1 : 0);
        return cudaSuccess;
    }
    // resident CTAs per SM of this instantiation, per device (a cooperative launch must not
    // exceed it)
    constexpr int kMaxDev = 64;
    static int blocks_per_sm[kMaxDev] = {};
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
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
    if (bp.prof && (e = cudaMemsetAsync(&bp.prof->exits, 0, sizeof(bp.prof->exits), stream)) != cudaSuccess) return e;
    e = cudaLaunchKernelEx(&cfg, batch_kernel<S>, bp);
    if (e == cudaSuccess) *launches += 1;
    return e;
}

}  // namespace

cudaError_t launch_batch(int shader, const BatchParams& bp, int form, int num_sms, cudaStream_t stream,
                         cudaEvent_t* phase_events, uint64_t* launches, bool clear_late) {
    switch (shader) {
        case kFlat: return launch_batch_s<kFlat>(bp, form, num_sms, stream, phase_events, launches, clear_late);
        case kPhong: return launch_batch_s<kPhong>(bp, form, num_sms, stream, phase_events, launches, clear_late);
        case kPBR: return launch_batch_s<kPBR>(bp, form, num_sms, stream, phase_events, launches, clear_late);
        case kBlinnPhong:
            return launch_batch_s<kBlinnPhong>(bp, form, num_sms, stream, phase_events, launches, clear_late);
        case kGouraud: return launch_batch_s<kGouraud>(bp, form, num_sms, stream, phase_events, launches, clear_late);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_merge_counters(DevCounters* dst, DevCounters* src, cudaStream_t stream) {
    merge_counters_kernel<<<1, 32, 0, stream>>>(dst, src);
    return cudaGetLastError();
}

cudaError_t launch_barrier_probe(DevCounters* counters, unsigned long long timeout_ns, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(counters, 0, kBatchCountersReset, stream);
    if (e != cudaSuccess) return e;
    barrier_probe_kernel<<<2, 32, 0, stream>>>(counters, timeout_ns);
    return cudaGetLastError();
}

}  // namespace axr
