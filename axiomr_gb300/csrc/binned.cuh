// Binned (sort-middle) form of a draw, shared by the per-draw kernels and the batched
// kernels (binned.cu). It follows the reference's tiled pipeline
// (src/tiled_pipeline.cpp:143-322): bin every triangle into the tiles its box covers
// (binTrianglesToTiles, cpp:368-393), rasterise each tile's list into a tile buffer of
// depth and colour (processTile / rasterizeTriangleInTile, cpp:395-594,
// include/tiled_pipeline.hpp:38-56) and merge the tile into the framebuffer once
// (mergeTileResults, cpp:1125-1181). On the GPU:
//
//   bin_face   one thread per face in draw order: clip classification, cull and edge setup
//              (the same device functions as the keyed form), the raster record at the
//              face's draw-order position, then one entry per bin of 8 tiles that the
//              triangle's box reaches and its edges do not provably miss. Bin slots come
//              from warp-aggregated atomics: the lanes of a warp that target the same bin
//              (neighbouring faces mostly do) take one atomicAdd between them.
//   bin_tile   one CTA per bin: depth keys of the bin's 2048 pixels in shared memory; the
//              bin's entries rasterised into them (small triangle-in-bin rectangles by one
//              thread each, larger ones by a whole warp), shared-memory atomicMin of
//              (depth, draw order) so the winner is the reference's sequential strict
//              early-Z winner whatever order the entries come in; the winners shaded with
//              the merge test against the framebuffer depth; colour and depth staged in
//              shared memory (loaded with TMA tensor loads when the draw does not clear the
//              plane) and written once per 16x16 tile with TMA tensor stores.
//
// Capacities only trade memory for speed: a bin offered more entries than its capacity,
// or a clipped triangle that finds the clipped-record list full, is rasterised by its own
// thread into the framebuffer's key plane (the keyed form's visibility keys) and marks the
// tiles it touched; the bin kernel folds those keys into its own before choosing winners.
#pragma once
#include <cuda_runtime.h>

#include "batch_types.h"
#include "draw_body.cuh"
#include "tma.cuh"

namespace axr {
namespace {

constexpr unsigned kFullMask = 0xFFFFFFFFu;
constexpr int kBinThreads = 256;  // one thread per pixel of a 16x16 tile
static_assert(kBinThreads == kTile * kTile, "a bin kernel thread owns one pixel of every tile of its bin");

struct PixRect {
    int x0, y0, x1, y1;  // pixels [x0, x1) x [y0, y1)
};

// Bin (bx, by) of the draw's target, clipped to the target.
__device__ __forceinline__ PixRect bin_rect(const DrawParams& p, int bx, int by) {
    const int bw = kTile * (int)p.bins.tw, bh = kTile * (int)p.bins.th;
    PixRect r;
    r.x0 = bx * bw;
    r.y0 = by * bh;
    r.x1 = min(r.x0 + bw, p.target.width);
    r.y1 = min(r.y0 + bh, p.target.height);
    return r;
}

// Whether no pixel of [x0, x1) x [y0, y1) (inside the triangle's box) can test covered:
// the argument of tile_outside (draw_body.cuh) over any rectangle. Each pixel is evaluated
// from a row start at most 15 columns to its left, so M = |a|(|x|+16) + |b||y| + |c| bounds
// the magnitudes of the terms of every evaluation in the rectangle.
__device__ __forceinline__ bool rect_outside(const Edges& e, int x0, int x1, int y0, int y1) {
    const float fx0 = (float)x0 + 0.5f, fx1 = (float)x1 - 0.5f;
    const float fy0 = (float)y0 + 0.5f, fy1 = (float)y1 - 0.5f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = e.a[k], b = e.b[k], c = e.c[k];
        const float ex = a >= 0.f ? a * fx1 : a * fx0;  // the larger of a*fx0, a*fx1
        const float ey = b >= 0.f ? b * fy1 : b * fy0;
        const float emax = (ex + ey) + c;
        const float m = fabsf(a) * (fabsf(fx1) + 16.0f) + fabsf(b) * fabsf(fy1) + fabsf(c);
        if (emax < -64.0f * 5.9604645e-8f * m) return true;
    }
    return false;
}

// Key slot of pixel (px, py) in a bin whose origin is (X0, Y0): tile-major, 256 per tile.
__device__ __forceinline__ int bin_slot(int px, int py, int X0, int Y0, int tw) {
    const int lx = px - X0, ly = py - Y0;
    return (((ly >> 4) * tw + (lx >> 4)) << 8) + ((ly & 15) << 4) + (lx & 15);
}

// Minimum of a shared-memory key and v (PTX red.shared.min.u64 on the shared-window
// address), skipped when v cannot win: keys only decrease, so a stale read is never below
// the current value.
__device__ __forceinline__ void key_min(unsigned long long* k, unsigned long long v) {
    const uint32_t a = smem_addr(k);
    unsigned long long cur;
    asm volatile("ld.volatile.shared.u64 %0, [%1];" : "=l"(cur) : "r"(a) : "memory");
    if (v < cur) asm volatile("red.shared.min.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}

// ------------------------------------------------------------------ rasterisation
// Coverage and depth over the rectangle [x0, x1) x [y0, y1) of the triangle's box, in this
// thread, with raster_box's arithmetic (per 16-pixel tile column the row start at the
// reference's column sx = max(tile start, x_lo), its 8-pixel step, then a*lane), into the
// bin's shared keys.
__device__ __forceinline__ void raster_rect_thread(const Edges& e, uint32_t tag, const PixRect& r, int X0, int Y0, int tw,
                                   unsigned long long* keys, uint32_t& frags, uint32_t& tested) {
    for (int tx = r.x0 >> 4; tx <= (r.x1 - 1) >> 4; ++tx) {
        const int cx0 = max(tx * kTile, r.x0), cx1 = min(tx * kTile + kTile, r.x1);
        const int sx = max(tx * kTile, e.x_lo);
        const float fsx = fadd((float)sx, 0.5f);
        float as[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) as[k] = fmul(e.a[k], fsx);
        for (int py = r.y0; py < r.y1; ++py) {
            const float fpy = fadd((float)py, 0.5f);
            float r0[3], r8[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                r0[k] = fadd(fadd(as[k], fmul(e.b[k], fpy)), e.c[k]);
                r8[k] = fadd(r0[k], fmul(e.a[k], 8.0f));
            }
            tested += (uint32_t)(cx1 - cx0);
            for (int px = cx0; px < cx1; ++px) {
                const int i = px - sx;
                const float lane = (float)(i & 7);
                float cov[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) cov[k] = fadd(i >= 8 ? r8[k] : r0[k], fmul(e.a[k], lane));
                if (cov[0] >= 0.f && cov[1] >= 0.f && cov[2] >= 0.f) {
                    ++frags;
                    const float al = fmul(cov[0], e.inv_area), be = fmul(cov[1], e.inv_area),
                                ga = fmul(cov[2], e.inv_area);
                    const float z = fadd(fadd(fmul(e.z[0], al), fmul(e.z[1], be)), fmul(e.z[2], ga));
                    if (z < __int_as_float(0x7f800000))  // +inf and NaN never pass early-Z
                        key_min(&keys[bin_slot(px, py, X0, Y0, tw)], make_key(z, tag));
                }
            }
        }
    }
}

// Smallest power of two >= v (v >= 1).
__device__ __forceinline__ int pow2_ceil(int v) { return v <= 1 ? 1 : 1 << (32 - __clz(v - 1)); }

// The same over a rectangle by a group of G threads (a warp: G = 32; the CTA: G = 256),
// `t` the thread's index in the group. The group covers wp = min(G, next power of two >=
// width) columns and G / wp rows at a time, so neighbouring threads touch neighbouring keys;
// a thread's column terms of eval_pixel (a*(sx+0.5) at the reference's row start sx, a*8,
// a*(offset in the 8-pixel block)) are computed once per column, then each row costs
// b*(y+0.5) and the adds, in eval_pixel's order.
template <int G>
__device__ __forceinline__ void raster_rect_group(const Edges& e, uint32_t tag, const PixRect& r, int X0, int Y0,
                                                  int tw, unsigned long long* keys, int t, uint32_t& frags,
                                                  uint32_t& tested) {
    const int wp = min(G, pow2_ceil(r.x1 - r.x0));
    const int col = t & (wp - 1), row0 = t / wp, rpp = G / wp;
    for (int xs = r.x0; xs < r.x1; xs += wp) {
        const int px = xs + col;
        if (px >= r.x1) continue;
        const int sx = max(px & ~(kTile - 1), e.x_lo);
        const int i = px - sx;
        const float fsx = fadd((float)sx, 0.5f), fl = (float)(i & 7);
        const bool hi = i >= 8;
        float as[3], al[3], a8[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            as[k] = fmul(e.a[k], fsx);
            al[k] = fmul(e.a[k], fl);
            a8[k] = fmul(e.a[k], 8.0f);
        }
        for (int py = r.y0 + row0; py < r.y1; py += rpp) {
            ++tested;
            const float fpy = fadd((float)py, 0.5f);
            float cov[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float row = fadd(fadd(as[k], fmul(e.b[k], fpy)), e.c[k]);
                if (hi) row = fadd(row, a8[k]);
                cov[k] = fadd(row, al[k]);
            }
            if (cov[0] >= 0.f && cov[1] >= 0.f && cov[2] >= 0.f) {
                ++frags;
                const float al_ = fmul(cov[0], e.inv_area), be = fmul(cov[1], e.inv_area),
                            ga = fmul(cov[2], e.inv_area);
                const float z = fadd(fadd(fmul(e.z[0], al_), fmul(e.z[1], be)), fmul(e.z[2], ga));
                if (z < __int_as_float(0x7f800000)) key_min(&keys[bin_slot(px, py, X0, Y0, tw)], make_key(z, tag));
            }
        }
    }
}

// ------------------------------------------------------------------ binning (face kernel)
// Spill of a (triangle, rectangle) pair that found no room: rasterised here into the key
// plane (write_key, as the keyed form does), the rectangle's tiles marked for the bin pass.
__device__ void spill_rect(const DrawParams& p, const BinSet& bs, const Edges& e, uint32_t tag, const PixRect& r,
                           GeomStats& st) {
    bool wrote = false;
    for (int py = r.y0; py < r.y1; ++py) {
        st.tested += (uint32_t)(r.x1 - r.x0);
        for (int px = r.x0; px < r.x1; ++px) {
            const PixelEval pe = eval_pixel(e, px, py);
            if (pe.covered) {
                ++st.frags;
                wrote |= write_key(p.target, px, py, pe.z, tag);
            }
        }
    }
    if (wrote)
        for (int ty = r.y0 >> 4; ty <= (r.y1 - 1) >> 4; ++ty)
            for (int tx = r.x0 >> 4; tx <= (r.x1 - 1) >> 4; ++tx)
                mark_tile(p.target, (uint32_t)ty * (uint32_t)p.target.tiles_x + (uint32_t)tx);
    atomicAdd(&bs.counters->spill, 1u);
}

// Cursor over the bins of a triangle's pixel box, row by row, skipping bins whose part of
// the box its edges provably miss.
struct BinCursor {
    int bx, by, bx0, bx1, by1;
    bool live;
};

__device__ __forceinline__ PixRect cursor_rect(const DrawParams& p, const Edges& e, const BinCursor& c) {
    PixRect r = bin_rect(p, c.bx, c.by);
    r.x0 = max(r.x0, e.x_lo);
    r.x1 = min(r.x1, e.x_hi);
    r.y0 = max(r.y0, e.y_lo);
    r.y1 = min(r.y1, e.y_hi);
    return r;
}

__device__ __forceinline__ void cursor_seek(const DrawParams& p, const Edges& e, BinCursor& c) {
    while (c.live) {
        if (c.by > c.by1) {
            c.live = false;
            return;
        }
        const PixRect r = cursor_rect(p, e, c);
        if (!rect_outside(e, r.x0, r.x1, r.y0, r.y1)) return;
        if (++c.bx > c.bx1) {
            c.bx = c.bx0;
            ++c.by;
        }
    }
}

__device__ __forceinline__ void cursor_start(const DrawParams& p, const Edges& e, bool live, BinCursor& c) {
    c.live = live;
    if (!live) return;
    const int sx = 4 + __ffs((int)p.bins.tw) - 1, sy = 4 + __ffs((int)p.bins.th) - 1;  // log2 of the bin size
    c.bx0 = e.x_lo >> sx;
    c.bx1 = (e.x_hi - 1) >> sx;
    c.by = e.y_lo >> sy;
    c.by1 = (e.y_hi - 1) >> sy;
    c.bx = c.bx0;
    if (c.bx0 != c.bx1 || c.by != c.by1) cursor_seek(p, e, c);  // one bin: no test needed
}

__device__ __forceinline__ void cursor_next(const DrawParams& p, const Edges& e, BinCursor& c) {
    if (++c.bx > c.bx1) {
        c.bx = c.bx0;
        ++c.by;
    }
    cursor_seek(p, e, c);
}

// Every lane's triangle (has = false: none) into its bins. All 32 lanes call it.
__device__ void bin_emit_warp(const DrawParams& p, const BinSet& bs, bool has, const Edges& e, uint32_t entry,
                              uint32_t tag, GeomStats& st) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const DevBins& b = p.bins;
    BinCursor c;
    cursor_start(p, e, has, c);
    while (__any_sync(kFullMask, c.live)) {
        const uint32_t lb = c.live ? (uint32_t)c.by * (uint32_t)b.bins_x + (uint32_t)c.bx : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(kFullMask, lb);
        if (c.live) {
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&bs.count[b.base + lb], (uint32_t)__popc(peers));
            base = __shfl_sync(peers, base, leader);
            const uint32_t slot = base + (uint32_t)__popc(peers & below);
            if (slot < b.cap)
                b.entries[(size_t)lb * b.cap + slot] = entry;
            else
                spill_rect(p, bs, e, tag, cursor_rect(p, e, c), st);
            cursor_next(p, e, c);
        }
    }
}

// One thread's triangle into its bins (clipped triangles: rare, not aggregated).
__device__ void bin_emit_thread(const DrawParams& p, const BinSet& bs, const Edges& e, uint32_t entry, uint32_t tag,
                                GeomStats& st) {
    const DevBins& b = p.bins;
    BinCursor c;
    cursor_start(p, e, true, c);
    while (c.live) {
        const uint32_t lb = (uint32_t)c.by * (uint32_t)b.bins_x + (uint32_t)c.bx;
        const uint32_t slot = atomicAdd(&bs.count[b.base + lb], 1u);
        if (slot < b.cap)
            b.entries[(size_t)lb * b.cap + slot] = entry;
        else
            spill_rect(p, bs, e, tag, cursor_rect(p, e, c), st);
        cursor_next(p, e, c);
    }
}

// A face that straddles the clip volume: the clipper's output triangles, each with a
// clipped raster record (tag = position * 16 + 8 + its index) and its bins.
__device__ __noinline__ void bin_clipped(const DrawParams& p, const BinSet& bs, uint32_t o, const uint3 f,
                                         GeomStats& st) {
    CVClip a[kMaxClipVerts], b[kMaxClipVerts];
    a[0].clip = load_clip(p.mesh, p.u.mvp, f.x);
    a[1].clip = load_clip(p.mesh, p.u.mvp, f.y);
    a[2].clip = load_clip(p.mesh, p.u.mvp, f.z);
    CVClip* out;
    const int n = clip_triangle<0>(a, b, &out);
    for (int j = 0; 3 * j + 2 < n; ++j) {
        Screen s;
        screen_setup(out[3 * j].clip, out[3 * j + 1].clip, out[3 * j + 2].clip, p.target.width, p.target.height, s);
        if (is_backface(s)) continue;
        ++st.tris;
        Edges e;
        if (!edge_setup(s, p.target.width, p.target.height, e)) continue;
        const uint32_t tag = (o << 4) | 8u | (uint32_t)j;
        const uint32_t slot = atomicAdd(&bs.counters->crec_count, 1u);
        if (slot < bs.crec_cap) {
            store_raster(bs.crec + (size_t)kRasterRec * slot, e, tag);
            bin_emit_thread(p, bs, e, kClipEntry | slot, tag, st);
        } else {
            if (raster_box(p.target, e, tag, st)) mark_box(p.target, e);
            atomicAdd(&bs.counters->spill, 1u);
        }
    }
}

// Face at draw-order position o (valid: o < num_drawn) of the binned form. All 32 lanes of
// the warp call it.
__device__ __forceinline__ void bin_face(const DrawParams& p, const BinSet& bs, uint32_t o, bool valid,
                                         DevCounters* counters, bool stats) {
    GeomStats st = {0, 0, 0, 0};
    bool has = false;
    Edges e;
    uint32_t tag = 0;
    if (valid) {
        if (o > kMaxOrdinal) {
            atomicOr(&counters->error, kErrOrdinal);
        } else {
            const FaceRef fr = face_of(p.mesh, o);
            const uint3 f = load_face(p.mesh, fr.face);
            const uint32_t nv = p.mesh.num_vertices;
            if (f.x >= nv || f.y >= nv || f.z >= nv) {
                atomicOr(&counters->error, kErrIndex);
            } else {
                const float4* vs = p.scratch.vscreen;
                const float4 g0 = __ldg(&vs[f.x]), g1 = __ldg(&vs[f.y]), g2 = __ldg(&vs[f.z]);
                const int cls = classify_masks(__float_as_uint(g0.w), __float_as_uint(g1.w), __float_as_uint(g2.w));
                if (cls == 3) {
                    Screen s;
                    s.x[0] = g0.x; s.y[0] = g0.y; s.z[0] = g0.z;
                    s.x[1] = g1.x; s.y[1] = g1.y; s.z[1] = g1.z;
                    s.x[2] = g2.x; s.y[2] = g2.y; s.z[2] = g2.z;
                    screen_bbox(s);
                    if (!is_backface(s)) {
                        ++st.tris;
                        if (edge_setup(s, p.target.width, p.target.height, e)) {
                            has = true;
                            tag = (o << 4) | kRecTag;
                            store_record(p, o, e, fr.material, f);
                        }
                    }
                } else if (cls < 0) {
                    bin_clipped(p, bs, o, f, st);
                }
            }
        }
    }
    bin_emit_warp(p, bs, has, e, o, tag, st);
    if (stats) {
        const uint32_t tr = __reduce_add_sync(kFullMask, st.tris), fr = __reduce_add_sync(kFullMask, st.frags);
        const uint32_t te = __reduce_add_sync(kFullMask, st.tested);
        if ((threadIdx.x & 31) == 0) {
            if (tr) atomicAdd(&counters->stat_triangles, (unsigned long long)tr);
            if (fr) atomicAdd(&counters->stat_fragments, (unsigned long long)fr);
            if (te) atomicAdd(&counters->stat_tested, (unsigned long long)te);
        }
    }
}

// ------------------------------------------------------------------ the bin pass
struct BinSmem {
    unsigned long long key[kBinTiles][256];  // depth keys of the bin's pixels
    __align__(128) uint32_t col[kBinTiles][256];  // colour staging, one 16x16 TMA box per tile
    __align__(128) float dep[kBinTiles][256];     // depth staging
    uint32_t wide[2][kBinThreads];                // entries left to the warp (front) and CTA (back)
                                                  // rasterisers, by round parity
    uint16_t wl[kBinThreads / 32][kBinTiles * 32]; // each warp's winners: tile << 8 | pixel
    uint32_t tile_has;                            // bit k: tile k has a winner
    uint32_t n_med[3], n_big[3];                  // queue fills, by round modulo 3
    uint32_t grab[2];                             // next warp-sized entry to hand out, by round parity
    uint32_t ok;
    uint64_t bar;                                 // arrival of the tile loads
};

// Raster record of a bin entry and the depth-key tag of its triangle.
__device__ __forceinline__ uint32_t load_entry(const DrawParams& p, const BinSet& bs, uint32_t entry, Edges& e) {
    if (entry & kClipEntry) {
        const float4* r = bs.crec + (size_t)kRasterRec * (entry & ~kClipEntry);
        return unpack_raster(__ldg(r), __ldg(r + 1), __ldg(r + 2), __ldg(r + 3), e);
    }
    const float4* r = p.scratch.rec + (size_t)kRecFloat4 * entry;
    unpack_raster(__ldg(r), __ldg(r + 1), __ldg(r + 2), __ldg(r + 3), e);
    return (entry << 4) | kRecTag;
}

__device__ __forceinline__ PixRect clip_rect(const PixRect& bin, const Edges& e) {
    return PixRect{max(bin.x0, e.x_lo), max(bin.y0, e.y_lo), min(bin.x1, e.x_hi), min(bin.y1, e.y_hi)};
}

// Both planes (or the requested ones) of a bin without entries set to the clear values.
__device__ void clear_bin(const DevTarget& t, const PixRect& R, bool cc, bool cd, uint32_t bgra, float depth) {
    const int rw = R.x1 - R.x0, rh = R.y1 - R.y0;
    if ((t.width & 3) == 0) {  // rows start 16-byte aligned: 4 pixels per store
        const int n4 = (rw + 3) >> 2;
        const uint4 c4 = make_uint4(bgra, bgra, bgra, bgra);
        const float4 d4 = make_float4(depth, depth, depth, depth);
        for (int i = threadIdx.x; i < n4 * rh; i += blockDim.x) {
            const int row = i / n4, q = i - row * n4;
            const int px = R.x0 + 4 * q;
            const size_t idx = (size_t)(R.y0 + row) * (size_t)t.width + (size_t)px;
            if (px + 4 <= R.x1) {
                if (cc) *reinterpret_cast<uint4*>(t.color + idx) = c4;
                if (cd) *reinterpret_cast<float4*>(t.depth + idx) = d4;
            } else {
                for (int k = 0; px + k < R.x1; ++k) {
                    if (cc) t.color[idx + k] = bgra;
                    if (cd) t.depth[idx + k] = depth;
                }
            }
        }
        return;
    }
    for (int i = threadIdx.x; i < rw * rh; i += blockDim.x) {
        const int row = i / rw, px = R.x0 + (i - row * rw);
        const size_t idx = (size_t)(R.y0 + row) * (size_t)t.width + (size_t)px;
        if (cc) t.color[idx] = bgra;
        if (cd) t.depth[idx] = depth;
    }
}

// The bin pass over local bin `lb` of the draw (bins of tw x th tiles, at most kBinTiles).
// `cmap`/`dmap`: tensor maps of the colour and depth planes (used when flags has kBatchTma);
// flags kBatchClearColor/Depth: the plane is cleared to clear_bgra / clear_depth before the
// draw (fused here), otherwise its tile contents are loaded and merged into. All threads of
// the CTA call it. Thread t owns pixel t of every tile of the bin in the key set-up, the
// winner scan and the plain (tensor-map-less) loads and stores.
template <int S>
__device__ void bin_tile(const DrawParams& p, const BinSet& bs, uint32_t lb, const TensorMap128* cmap,
                         const TensorMap128* dmap, uint32_t flags, uint32_t clear_bgra, float clear_depth, BinSmem& sm,
                         DevCounters* counters, bool stats) {
    const DevTarget& t = p.target;
    const DevBins& b = p.bins;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tw = (int)b.tw, nt = (int)b.tw * (int)b.th;
    const int bx = (int)(lb % (uint32_t)b.bins_x), by = (int)(lb / (uint32_t)b.bins_x);
    const PixRect R = bin_rect(p, bx, by);
    const uint32_t offered = *reinterpret_cast<const volatile uint32_t*>(&bs.count[b.base + lb]);
    const uint32_t n = min(offered, b.cap);
    const bool clear_c = (flags & kBatchClearColor) != 0u, clear_d = (flags & kBatchClearDepth) != 0u;
    // tile k of the bin has its origin at tile_x(k), tile_y(k); it exists when that lies
    // inside the target
    auto tile_x = [&](int k) { return R.x0 + kTile * (k % tw); };
    auto tile_y = [&](int k) { return R.y0 + kTile * (k / tw); };
    // whether a tile of this bin holds spilled keys (only looked at when the launch spilled)
    bool spilled = false;
    if (*reinterpret_cast<const volatile uint32_t*>(&bs.counters->spill) != 0u) {
        bool flag = false;
        if (tid < nt && tile_x(tid) < t.width && tile_y(tid) < t.height)
            flag = ld_volatile(&t.tile_flag[(uint32_t)(tile_y(tid) >> 4) * (uint32_t)t.tiles_x +
                                            (uint32_t)(tile_x(tid) >> 4)]) != 0u;
        spilled = __syncthreads_or(flag) != 0;
    }
    if (n == 0 && !spilled) {
        if (clear_c || clear_d) clear_bin(t, R, clear_c, clear_d, clear_bgra, clear_depth);
        return;
    }
    const bool tma = (flags & kBatchTma) != 0u;
    const bool load_c = !clear_c, load_d = !clear_d;
    const uint32_t* list = b.entries + (size_t)lb * b.cap;
    uint32_t next = (uint32_t)tid < n ? __ldg(list + tid) : 0u;  // round 0's entry, in flight during set-up
    if (tid == 0) {
        sm.n_med[0] = sm.n_med[1] = 0u;
        sm.n_big[0] = sm.n_big[1] = 0u;
        sm.grab[0] = sm.grab[1] = 0u;
        sm.ok = 1u;
        sm.tile_has = 0u;
        mbar_init(&sm.bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0 && tma && (load_c || load_d)) {
        uint32_t bytes = 0;
        for (int k = 0; k < nt; ++k)
            if (tile_x(k) < t.width && tile_y(k) < t.height) bytes += (load_c ? 1024u : 0u) + (load_d ? 1024u : 0u);
        mbar_arrive_expect_tx(&sm.bar, bytes);
        for (int k = 0; k < nt; ++k) {
            const int x = tile_x(k), y = tile_y(k);
            if (x >= t.width || y >= t.height) continue;
            if (load_c) tma_load_tile(cmap, sm.col[k], &sm.bar, x, y);
            if (load_d) tma_load_tile(dmap, sm.dep[k], &sm.bar, x, y);
        }
    }
    const int lx = tid & 15, ly = tid >> 4;  // this thread's pixel in every tile
    for (int k = 0; k < nt; ++k) {
        sm.key[k][tid] = kEmptyKey;
        if (!tma && (load_c || load_d)) {  // no tensor maps: plain loads
            const int px = tile_x(k) + lx, py = tile_y(k) + ly;
            if (px < t.width && py < t.height) {
                const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
                if (load_c) sm.col[k][tid] = t.color[idx];
                if (load_d) sm.dep[k][tid] = t.depth[idx];
            }
        }
    }
    __syncthreads();

    // ---- rasterise the bin's entries, kBinThreads per round. A triangle's part of the bin
    // of at most thread_px pixels is rasterised by its thread, up to 256 pixels by a warp,
    // larger by the whole CTA. One barrier per round: the queues alternate between two
    // buffers (warp entries from the front, CTA entries from the back), their fill counters
    // among three (round r clears the counters of round r + 2 after its barrier).
    uint32_t frags = 0, tested = 0, wides = 0;
    unsigned long long* keys = &sm.key[0][0];
    uint32_t round = 0;
    for (uint32_t base = 0; base < n; base += kBinThreads, ++round) {
        const uint32_t q = base + (uint32_t)tid;
        const uint32_t entry = next;
        if (q + kBinThreads < n) next = __ldg(list + q + kBinThreads);
        if (q < n) {
            Edges e;
            const uint32_t tag = load_entry(p, bs, entry, e);
            const PixRect r = clip_rect(R, e);
            if (r.x0 < r.x1 && r.y0 < r.y1) {
                const int npx = (r.x1 - r.x0) * (r.y1 - r.y0);
                if (npx <= (int)b.thread_px)
                    raster_rect_thread(e, tag, r, R.x0, R.y0, tw, keys, frags, tested);
                else if (npx <= 256)
                    sm.wide[round & 1][atomicAdd(&sm.n_med[round % 3], 1u)] = entry;
                else
                    sm.wide[round & 1][kBinThreads - 1 - atomicAdd(&sm.n_big[round % 3], 1u)] = entry;
            }
        }
        __syncthreads();
        const uint32_t nm = sm.n_med[round % 3], nb = sm.n_big[round % 3];
        if (tid == 0) {
            sm.n_med[(round + 2) % 3] = sm.n_big[(round + 2) % 3] = 0u;
            sm.grab[(round + 1) & 1] = 0u;  // last used in round r - 1, whose grabs ended before this barrier
        }
        wides += nm + nb;
        // CTA-wide triangles first (every warp takes part in each), then the warp-sized ones
        // handed out one at a time to whichever warp is free
        for (uint32_t k = 0; k < nb; ++k) {
            const uint32_t we = sm.wide[round & 1][kBinThreads - 1 - k];
            Edges e;
            const uint32_t tag = load_entry(p, bs, we, e);
            raster_rect_group<kBinThreads>(e, tag, clip_rect(R, e), R.x0, R.y0, tw, keys, tid, frags, tested);
        }
        for (;;) {
            uint32_t k = 0;
            if (lane == 0) k = atomicAdd(&sm.grab[round & 1], 1u);
            k = __shfl_sync(kFullMask, k, 0);
            if (k >= nm) break;
            const uint32_t we = sm.wide[round & 1][k];
            Edges e;
            const uint32_t tag = load_entry(p, bs, we, e);
            raster_rect_group<32>(e, tag, clip_rect(R, e), R.x0, R.y0, tw, keys, lane, frags, tested);
        }
    }
    __syncthreads();

    // ---- winners, per warp: keys spilled into the key plane folded in first, then the warp's
    // winner pixels (its two rows of every tile: coverage spreads evenly over the warps)
    // compacted by ballots into its own list and shaded by the warp
    const unsigned below = (1u << lane) - 1u;
    uint32_t nw = 0;  // winners of this warp
    for (int k = 0; k < nt; ++k) {
        const int ox = tile_x(k), oy = tile_y(k), px = ox + lx, py = oy + ly;
        const bool in = ox < t.width && oy < t.height && px < t.width && py < t.height;
        unsigned long long key = sm.key[k][tid];
        if (spilled && in) {
            const uint32_t tile = (uint32_t)(oy >> 4) * (uint32_t)t.tiles_x + (uint32_t)(ox >> 4);
            if (ld_volatile(&t.tile_flag[tile]) != 0u) {
                const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
                const unsigned long long g = t.key[idx];
                if (g != kEmptyKey) {
                    key = g < key ? g : key;
                    sm.key[k][tid] = key;
                    t.key[idx] = kEmptyKey;  // the key plane is all-ones between draws
                }
            }
        }
        const bool has = in && key != kEmptyKey;
        const unsigned m = __ballot_sync(kFullMask, has);
        if (has) sm.wl[warp][nw + (uint32_t)__popc(m & below)] = (uint16_t)((k << 8) | tid);
        nw += (uint32_t)__popc(m);
        if (m && lane == 0) atomicOr(&sm.tile_has, 1u << k);
        if (clear_c) sm.col[k][tid] = clear_bgra;
        if (clear_d) sm.dep[k][tid] = clear_depth;
    }
    // the loaded planes must have arrived before the merge test reads them
    bool loaded = true;
    if (tma && (load_c || load_d) && !mbar_wait_bounded(&sm.bar, 0)) {
        atomicOr(&counters->error, kErrTma);
        sm.ok = 0u;
        loaded = false;
    }
    __syncwarp();
    for (uint32_t q = (uint32_t)lane; loaded && q < nw; q += 32) {
        const uint32_t v = sm.wl[warp][q];
        const int k = (int)(v >> 8);
        const uint32_t pix = v & 255u;
        const uint32_t tag = (uint32_t)sm.key[k][pix];
        const int gx = tile_x(k) + (int)(pix & 15u), gy = tile_y(k) + (int)(pix >> 4);
        const float old = clear_d ? clear_depth : sm.dep[k][pix];
        uint32_t bgra = 0u;
        float z = 0.0f;
        const bool ok = (tag & 8u) ? shade_clipped_px<S>(p, tag, gx, gy, old, &bgra, &z)
                                   : shade_unclipped<S, false>(p, tag, gx, gy, old, bgra, z);
        if (ok) {
            sm.col[k][pix] = bgra;
            sm.dep[k][pix] = z;
        }
    }
    if (stats) {
        const uint32_t f = __reduce_add_sync(kFullMask, frags), te = __reduce_add_sync(kFullMask, tested);
        if (lane == 0) {
            if (f) atomicAdd(&counters->stat_fragments, (unsigned long long)f);
            if (te) atomicAdd(&counters->stat_tested, (unsigned long long)te);
            if (nw) atomicAdd(&counters->stat_shaded, (unsigned long long)nw);
        }
        if (tid == 0) {
            atomicAdd(&counters->stat_tiles, 1ull);
            if (wides) atomicAdd(&counters->stat_large, (unsigned long long)wides);
        }
    }
    __syncthreads();
    if (spilled && tid < nt) {  // flags of the folded tiles back to zero (after every read)
        const int ox = tile_x(tid), oy = tile_y(tid);
        if (ox < t.width && oy < t.height) t.tile_flag[(uint32_t)(oy >> 4) * (uint32_t)t.tiles_x + (uint32_t)(ox >> 4)] = 0u;
    }
    if (!sm.ok) {  // tile contents unknown: leave the framebuffer as it is
        // the CTA's shared memory outlives loads still in flight only while a thread stays:
        // one more bounded wait for them before the CTA exits
        if (tid == 0) mbar_wait_bounded(&sm.bar, 0);
        return;
    }
    const uint32_t tile_has = sm.tile_has;

    // ---- write the tiles out: a plane of a tile is written when it was cleared or the tile
    // has winners
    if (tma) {
        tma_fence_smem();
        __syncthreads();
        if (tid == 0) {
            for (int k = 0; k < nt; ++k) {
                const int x = tile_x(k), y = tile_y(k);
                if (x >= t.width || y >= t.height) continue;
                const bool any = (tile_has >> k) & 1u;
                if (clear_c || any) tma_store_tile(cmap, sm.col[k], x, y);
                if (clear_d || any) tma_store_tile(dmap, sm.dep[k], x, y);
            }
            tma_commit();
            tma_wait_read_0();  // shared memory is released when the CTA exits
        }
        return;
    }
    __syncthreads();
    for (int k = 0; k < nt; ++k) {
        const int px = tile_x(k) + lx, py = tile_y(k) + ly;
        if (px >= t.width || py >= t.height) continue;
        const size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
        const bool any = (tile_has >> k) & 1u;
        if (clear_c || any) t.color[idx] = sm.col[k][tid];
        if (clear_d || any) t.depth[idx] = sm.dep[k][tid];
    }
}

}  // namespace
}  // namespace axr
