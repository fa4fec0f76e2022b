// Draw kernels for sm_103a.
//
// A draw is a counter reset (memset) and six launches on one stream:
//   vertex_kernel    one thread per vertex: clip position (mvp * pos), screen position and
//                    NDC depth (the per-vertex part of the reference's Triangle ctor,
//                    src/tiled_pipeline.cpp:53-72), clip-plane masks, and the shader's
//                    vertex outputs (IShader::vertex, include/shaders/shaders.hpp). The
//                    reference recomputes these for every face a vertex belongs to (clip
//                    stage) and every tile a triangle touches (processTile, cpp:407-409);
//                    they depend only on the vertex, so one evaluation gives the same bits.
//   geometry_kernel  one thread per face in draw order: clip classification from the
//                    vertex masks (exact clipper for faces that straddle a plane), backface
//                    cull and edge setup (cpp:195-236, 436-487). Triangles whose pixel box
//                    is small are rasterised by the same thread; larger ones get one setup
//                    record and one work item per 16x16 tile of their box.
//   large_kernel     warps take tile work items (4 per atomic) and evaluate 256 pixels
//                    each, 8 per lane.
//   scan_kernel      one warp per flagged 16x16 tile: compacts the tile's covered pixels
//                    (non-empty depth keys) into the shade / clipped lists, resets the keys.
//   shade_kernel     one thread per covered pixel: the winner is re-derived from its depth
//                    key, shaded once, and merged into the framebuffer with the reference's
//                    strict less-than test (winners that were clipped go to
//                    resolve_clipped_kernel).
// Visibility is order independent: every covered pixel does a fire-and-forget 64-bit
// atomicMin of (depth, draw-order position), so the surviving key is the reference's
// early-Z winner (minimum depth, earliest triangle on ties) whatever order the threads
// run in. Only the winning fragment is shaded; the reference shades every fragment that
// passes its early test at the time, with the same final colour.
#include <cuda_runtime.h>

#include <cstddef>

#include "kernels.h"
#include "raster.cuh"
#include "shade.cuh"

namespace axr {

namespace {

constexpr int kBlock = 256;
constexpr uint32_t kNoTile = 0xFFFFFFFFu;

// Resident 256-thread CTAs per SM the geometry kernel is compiled for (register budget
// 65536 / (256 * n)); 5 keeps it at 48 registers.
#ifndef AXR_GEOMETRY_MIN_BLOCKS
#define AXR_GEOMETRY_MIN_BLOCKS 5
#endif

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) { return *reinterpret_cast<const volatile uint32_t*>(p); }

// A tile that holds at least one depth key is flagged for the key scan (a plain store:
// every writer stores the same value).
__device__ __forceinline__ void mark_tile(const DevTarget& t, uint32_t tile) { t.tile_flag[tile] = 1u; }

__device__ __forceinline__ uint32_t tile_of(const DevTarget& t, int px, int py) {
    return (uint32_t)(py >> 4) * (uint32_t)t.tiles_x + (uint32_t)(px >> 4);
}

// Visibility write of one covered pixel (no return value used: compiles to a reduction).
// Returns whether a key was written.
__device__ __forceinline__ bool write_key(const DevTarget& t, int px, int py, float z, uint32_t tag) {
    if (!(z < __int_as_float(0x7f800000))) return false;  // +inf and NaN never pass early-Z
    atomicMin(&t.key[(uint32_t)py * (uint32_t)t.width + (uint32_t)px], make_key(z, tag));
    return true;
}

struct GeomStats {
    uint32_t tris, frags, large;
};

// Rasterise a small triangle's pixel box in this thread; returns whether any key was
// written. Walks the box the way the reference's tile raster does: per 16-pixel tile
// column and row, the row start (a*(sx+0.5) + b*(py+0.5)) + c and its 8-pixel step are
// computed once, then each pixel adds a*lane (eval_pixel gives the same bits per pixel).
__device__ bool raster_box(const DevTarget& t, const Edges& e, uint32_t tag, GeomStats& st) {
    bool wrote = false;
    for (int tx = e.x_lo >> 4; tx <= (e.x_hi - 1) >> 4; ++tx) {
        const int sx = max(tx * kTile, e.x_lo);
        const int ex = min((tx + 1) * kTile, e.x_hi);
        const float fsx = fadd((float)sx, 0.5f);
        float as[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) as[k] = fmul(e.a[k], fsx);
        for (int py = e.y_lo; py < e.y_hi; ++py) {
            const float fpy = fadd((float)py, 0.5f);
            float r0[3], r8[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                r0[k] = fadd(fadd(as[k], fmul(e.b[k], fpy)), e.c[k]);
                r8[k] = fadd(r0[k], fmul(e.a[k], 8.0f));
            }
            for (int px = sx; px < ex; ++px) {
                const int i = px - sx;
                const float lane = (float)(i & 7);
                float cov[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) cov[k] = fadd(i >= 8 ? r8[k] : r0[k], fmul(e.a[k], lane));
                if (cov[0] >= 0.f && cov[1] >= 0.f && cov[2] >= 0.f) {
                    ++st.frags;
                    const float al = fmul(cov[0], e.inv_area), be = fmul(cov[1], e.inv_area),
                                ga = fmul(cov[2], e.inv_area);
                    const float z = fadd(fadd(fmul(e.z[0], al), fmul(e.z[1], be)), fmul(e.z[2], ga));
                    wrote |= write_key(t, px, py, z, tag);
                }
            }
        }
    }
    return wrote;
}

__device__ __forceinline__ uint32_t tiles_of(const Edges& e, uint32_t& ntx) {
    int tx0 = e.x_lo >> 4, tx1 = (e.x_hi - 1) >> 4;
    int ty0 = e.y_lo >> 4, ty1 = (e.y_hi - 1) >> 4;
    ntx = (uint32_t)(tx1 - tx0 + 1);
    return ntx * (uint32_t)(ty1 - ty0 + 1);
}

__device__ void mark_box(const DevTarget& t, const Edges& e) {
    for (int ty = e.y_lo >> 4; ty <= (e.y_hi - 1) >> 4; ++ty)
        for (int tx = e.x_lo >> 4; tx <= (e.x_hi - 1) >> 4; ++tx)
            mark_tile(t, (uint32_t)ty * (uint32_t)t.tiles_x + (uint32_t)tx);
}

__device__ __forceinline__ void store_large(LargeTri* dst, const Edges& e, uint32_t tag) {
    float4* d = reinterpret_cast<float4*>(dst);
    d[0] = make_float4(e.a[0], e.b[0], e.c[0], e.a[1]);
    d[1] = make_float4(e.b[1], e.c[1], e.a[2], e.b[2]);
    d[2] = make_float4(e.c[2], e.inv_area, e.z[0], e.z[1]);
    uint32_t xs = (uint32_t)e.x_lo | ((uint32_t)e.x_hi << 16);
    uint32_t ys = (uint32_t)e.y_lo | ((uint32_t)e.y_hi << 16);
    d[3] = make_float4(e.z[2], __uint_as_float(tag), __uint_as_float(xs), __uint_as_float(ys));
}

__device__ __forceinline__ void load_large(const LargeTri* src, Edges& e, uint32_t& tag) {
    const float4* s = reinterpret_cast<const float4*>(src);
    float4 v0 = s[0], v1 = s[1], v2 = s[2], v3 = s[3];
    e.a[0] = v0.x; e.b[0] = v0.y; e.c[0] = v0.z; e.a[1] = v0.w;
    e.b[1] = v1.x; e.c[1] = v1.y; e.a[2] = v1.z; e.b[2] = v1.w;
    e.c[2] = v2.x; e.inv_area = v2.y; e.z[0] = v2.z; e.z[1] = v2.w;
    e.z[2] = v3.x;
    tag = __float_as_uint(v3.y);
    uint32_t xs = __float_as_uint(v3.z), ys = __float_as_uint(v3.w);
    e.x_lo = (int)(xs & 0xFFFFu); e.x_hi = (int)(xs >> 16);
    e.y_lo = (int)(ys & 0xFFFFu); e.y_hi = (int)(ys >> 16);
}

// One triangle that survived clipping: cull, set up, then rasterise it here or queue its
// tiles. *single_tile receives the one tile a small triangle wrote to (the caller marks
// it after deduplicating across the warp); boxes spanning several tiles are marked here.
__device__ void emit_triangle(const DrawParams& p, const Screen& s, uint32_t tag, GeomStats& st,
                              uint32_t* single_tile) {
    if (is_backface(s)) return;
    ++st.tris;
    Edges e;
    if (!edge_setup(s, p.target.width, p.target.height, e)) return;
    const int npx = (e.x_hi - e.x_lo) * (e.y_hi - e.y_lo);
    DevCounters* c = p.scratch.counters;
    if (npx <= p.small_max_pixels) {
        if (raster_box(p.target, e, tag, st)) {
            uint32_t ntx;
            if (tiles_of(e, ntx) == 1u && *single_tile == kNoTile)
                *single_tile = tile_of(p.target, e.x_lo, e.y_lo);
            else
                mark_box(p.target, e);
        }
        return;
    }
    uint32_t ntx;
    const uint32_t nt = tiles_of(e, ntx);
    const uint32_t slot = atomicAdd(&c->large_count, 1u);
    const uint32_t base = atomicAdd(&c->item_count, nt);
    const uint32_t icap = p.scratch.item_cap;
    if (slot < p.scratch.large_cap && base + nt <= icap && base + nt > base) {
        store_large(&p.scratch.large[slot], e, tag);
        for (uint32_t k = 0; k < nt; ++k) p.scratch.items[base + k] = LargeItem{slot, k};
        ++st.large;
    } else {
        // lists full: mark the reserved items empty and rasterise the triangle here
        for (uint32_t k = base; k < icap && k - base < nt; ++k) p.scratch.items[k] = LargeItem{kNoItem, 0u};
        if (raster_box(p.target, e, tag, st)) mark_box(p.target, e);
    }
}

template <int S>
__global__ void __launch_bounds__(kBlock) vertex_kernel(const __grid_constant__ DrawParams p) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= p.mesh.num_vertices) return;
    constexpr int A = ShaderAttrs<S>::mask;
    CVFull v = load_vertex<A>(p.mesh, i);
    f4 clip = mat4_mul(p.u.mvp, v.pos.x, v.pos.y, v.pos.z, 1.0f);
    f3 sc = screen_vertex(clip, (float)p.target.width, (float)p.target.height);
    p.scratch.vscreen[i] = make_float4(sc.x, sc.y, sc.z, __uint_as_float(plane_masks(clip)));
    pack_vsout<S>(vertex_shader<S>(p.u, v), &p.scratch.vattr[(size_t)VAttr<S>::n * i]);
}

__global__ void __launch_bounds__(kBlock, AXR_GEOMETRY_MIN_BLOCKS) geometry_kernel(const __grid_constant__ DrawParams p) {
    GeomStats st = {0, 0, 0};
    uint32_t single_tile = kNoTile;
    const uint32_t o = blockIdx.x * kBlock + threadIdx.x;
    if (o < p.mesh.num_drawn) {
        if (o > kMaxOrdinal) {
            atomicOr(&p.scratch.counters->error, kErrOrdinal);
        } else {
            const FaceRef fr = face_of(p.mesh, o);
            const uint3 f = load_face(p.mesh, fr.face);
            const uint32_t nv = p.mesh.num_vertices;
            if (f.x >= nv || f.y >= nv || f.z >= nv) {
                atomicOr(&p.scratch.counters->error, kErrIndex);
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
                    emit_triangle(p, s, o << 4, st, &single_tile);
                } else if (cls < 0) {
                    CVClip a[kMaxClipVerts], b[kMaxClipVerts];
                    a[0].clip = load_clip(p.mesh, p.u.mvp, f.x);
                    a[1].clip = load_clip(p.mesh, p.u.mvp, f.y);
                    a[2].clip = load_clip(p.mesh, p.u.mvp, f.z);
                    CVClip* out;
                    const int n = clip_triangle<0>(a, b, &out);
                    for (int j = 0; 3 * j + 2 < n; ++j) {
                        Screen s;
                        screen_setup(out[3 * j].clip, out[3 * j + 1].clip, out[3 * j + 2].clip, p.target.width,
                                     p.target.height, s);
                        uint32_t tile = kNoTile;
                        emit_triangle(p, s, (o << 4) | 8u | (uint32_t)j, st, &tile);
                        if (tile != kNoTile) mark_tile(p.target, tile);
                    }
                }
            }
        }
    }
    // one mark per distinct tile in the warp
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, single_tile);
    if (single_tile != kNoTile && (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1))
        mark_tile(p.target, single_tile);
    if (p.scratch.collect_stats) {
        const unsigned full = 0xFFFFFFFFu;
        uint32_t t = __reduce_add_sync(full, st.tris), fr = __reduce_add_sync(full, st.frags);
        uint32_t l = __reduce_add_sync(full, st.large);
        if ((threadIdx.x & 31) == 0) {
            DevCounters* c = p.scratch.counters;
            if (t) atomicAdd(&c->stat_triangles, (unsigned long long)t);
            if (fr) atomicAdd(&c->stat_fragments, (unsigned long long)fr);
            if (l) atomicAdd(&c->stat_large, (unsigned long long)l);
        }
    }
}

__global__ void __launch_bounds__(kBlock) large_kernel(const __grid_constant__ DrawParams p) {
    DevCounters* c = p.scratch.counters;
    const uint32_t n_items = min(ld_volatile(&c->item_count), p.scratch.item_cap);
    if (n_items == 0) return;
    const uint32_t n_tris = min(ld_volatile(&c->large_count), p.scratch.large_cap);
    const int lane = threadIdx.x & 31;
    uint32_t frags = 0;
    for (;;) {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(&c->item_head, kItemsPerGrab);
        first = __shfl_sync(0xFFFFFFFFu, first, 0);
        if (first >= n_items) break;
        const uint32_t last = min(first + kItemsPerGrab, n_items);
        for (uint32_t it = first; it < last; ++it) {
            const LargeItem item = p.scratch.items[it];
            if (item.tri >= n_tris) continue;  // reserved slot of a triangle rasterised elsewhere
            Edges e;
            uint32_t tag;
            load_large(&p.scratch.large[item.tri], e, tag);
            uint32_t ntx;
            tiles_of(e, ntx);
            const int tx = (e.x_lo >> 4) + (int)(item.tile % ntx);
            const int ty = (e.y_lo >> 4) + (int)(item.tile / ntx);
            const int px = tx * kTile + (lane & 15);
            bool wrote = false;
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int py = ty * kTile + (lane >> 4) + 2 * r;
                if (px >= e.x_lo && px < e.x_hi && py >= e.y_lo && py < e.y_hi) {
                    PixelEval pe = eval_pixel(e, px, py);
                    if (pe.covered) {
                        ++frags;
                        wrote |= write_key(p.target, px, py, pe.z, tag);
                    }
                }
            }
            if (__any_sync(0xFFFFFFFFu, wrote) && lane == 0)
                mark_tile(p.target, (uint32_t)ty * (uint32_t)p.target.tiles_x + (uint32_t)tx);
        }
    }
    if (p.scratch.collect_stats) {
        uint32_t f = __reduce_add_sync(0xFFFFFFFFu, frags);
        if (lane == 0 && f) atomicAdd(&c->stat_fragments, (unsigned long long)f);
    }
}

// Key scan over every tile of the target, one warp per tile and 8 tiles per CTA round:
// flagged tiles have their 256 keys read (8 per lane), every covered pixel is appended as
// (pixel, tag) to the shade list, or to the clipped list when its winner came out of the
// clipper, and the keys and the flag are reset. List space is taken once per CTA round
// (shared-memory prefix over the 8 warps), so the global counters see few atomics.
__global__ void __launch_bounds__(kBlock) scan_kernel(const __grid_constant__ DrawParams p) {
    constexpr int kWarps = kBlock / 32;
    __shared__ uint32_t s_count[2][kWarps];
    __shared__ uint32_t s_base[2];
    DevCounters* c = p.scratch.counters;
    const DevTarget& t = p.target;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t ntiles = (uint32_t)t.tiles_x * (uint32_t)t.tiles_y;
    for (uint32_t first = blockIdx.x * kWarps; first < ntiles; first += gridDim.x * kWarps) {
        const uint32_t tile = first + (uint32_t)warp;
        const bool dirty = tile < ntiles && ld_volatile(&t.tile_flag[tile]) != 0u;
        const int px = (int)(tile % (uint32_t)t.tiles_x) * kTile + (lane & 15);
        const int py0 = (int)(tile / (uint32_t)t.tiles_x) * kTile + (lane >> 4);
        unsigned long long keys[8];
        unsigned ms[8], mc[8];
        uint32_t ns = 0, nc = 0;
        if (dirty) {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int py = py0 + 2 * r;
                keys[r] = (px < t.width && py < t.height) ? t.key[(uint32_t)py * (uint32_t)t.width + (uint32_t)px]
                                                          : kEmptyKey;
            }
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const bool has = keys[r] != kEmptyKey;
                const bool clipped = has && (((uint32_t)keys[r]) & 8u) != 0u;
                ms[r] = __ballot_sync(0xFFFFFFFFu, has && !clipped);
                mc[r] = __ballot_sync(0xFFFFFFFFu, clipped);
                ns += (uint32_t)__popc(ms[r]);
                nc += (uint32_t)__popc(mc[r]);
            }
        }
        if (lane == 0) {
            s_count[0][warp] = ns;
            s_count[1][warp] = nc;
        }
        __syncthreads();
        if (threadIdx.x < 2) {
            uint32_t total = 0;
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t v = s_count[threadIdx.x][w];
                s_count[threadIdx.x][w] = total;
                total += v;
            }
            s_base[threadIdx.x] = total ? atomicAdd(threadIdx.x == 0 ? &c->shade_count : &c->clip_count, total) : 0u;
        }
        __syncthreads();
        if (dirty) {
            uint32_t bs = s_base[0] + s_count[0][warp], bc = s_base[1] + s_count[1][warp];
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                if (keys[r] != kEmptyKey) {
                    const uint32_t idx = (uint32_t)(py0 + 2 * r) * (uint32_t)t.width + (uint32_t)px;
                    const uint2 entry = make_uint2(idx, (uint32_t)keys[r]);
                    if ((uint32_t)keys[r] & 8u)
                        p.scratch.clip_px[bc + (uint32_t)__popc(mc[r] & below)] = entry;
                    else
                        p.scratch.shade[bs + (uint32_t)__popc(ms[r] & below)] = entry;
                    t.key[idx] = kEmptyKey;
                }
                bs += (uint32_t)__popc(ms[r]);
                bc += (uint32_t)__popc(mc[r]);
            }
            if (lane == 0) {
                t.tile_flag[tile] = 0u;
                if (p.scratch.collect_stats) atomicAdd(&c->stat_tiles, 1ull);
            }
        }
        __syncthreads();
    }
}

// Shade a pixel's winner given its setup and vertex outputs; strict merge into the framebuffer.
template <int S>
__device__ __forceinline__ void shade_winner(const DrawParams& p, size_t idx, int px, int py, uint32_t material,
                                             Screen& s, const VSOut* vo) {
    const DevTarget& t = p.target;
    Edges e;
    if (!edge_setup(s, t.width, t.height, e)) return;
    const PixelEval r = eval_pixel(e, px, py);
    if (!(r.z < t.depth[idx])) return;  // merge: tile depth < framebuffer depth (strict)
    const f4 col = fragment_shader<S>(p.u, p.mesh.materials[material], mk3(r.alpha, r.beta, r.gamma), vo);
    t.color[idx] = pack_bgra(col);
    t.depth[idx] = r.z;
}

// Dense shading of the covered pixels whose winner is unclipped: the winner is re-derived
// from its tag (face -> cached vertex screen positions and shader outputs), its
// barycentrics recomputed exactly and the fragment shaded once.
template <int S>
__global__ void __launch_bounds__(kBlock) shade_kernel(const __grid_constant__ DrawParams p) {
    DevCounters* c = p.scratch.counters;
    const DevTarget& t = p.target;
    const uint32_t n = min(ld_volatile(&c->shade_count), p.scratch.px_cap);
    for (uint32_t q = blockIdx.x * kBlock + threadIdx.x; q < n; q += gridDim.x * kBlock) {
        const uint2 w = p.scratch.shade[q];
        const uint32_t tag = w.y;
        const size_t idx = w.x;
        const int px = (int)(idx % (size_t)t.width), py = (int)(idx / (size_t)t.width);
        const FaceRef fr = face_of(p.mesh, tag >> 4);
        const uint3 f = load_face(p.mesh, fr.face);
        Screen s;
        VSOut vo[3];
        const uint32_t vi[3] = {f.x, f.y, f.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float4 g = __ldg(&p.scratch.vscreen[vi[k]]);
            s.x[k] = g.x;
            s.y[k] = g.y;
            s.z[k] = g.z;
            vo[k] = unpack_vsout<S>(&p.scratch.vattr[(size_t)VAttr<S>::n * vi[k]]);
        }
        screen_bbox(s);
        shade_winner<S>(p, idx, px, py, fr.material, s, vo);
    }
}

// Pixels whose winner is a clipped triangle: re-run the clipper on the face's raw vertex
// attributes (the geometry stage's clip, now carrying attributes; src/pipeline.cpp:243-272)
// and take output triangle j of the tag.
template <int S>
__global__ void __launch_bounds__(kBlock) resolve_clipped_kernel(const __grid_constant__ DrawParams p) {
    const uint32_t n = min(ld_volatile(&p.scratch.counters->clip_count), p.scratch.px_cap);
    constexpr int A = ShaderAttrs<S>::mask;
    const DevTarget& t = p.target;
    for (uint32_t q = blockIdx.x * kBlock + threadIdx.x; q < n; q += gridDim.x * kBlock) {
        const uint2 w = p.scratch.clip_px[q];
        const size_t idx = w.x;
        const uint32_t tag = w.y;
        const int px = (int)(idx % (size_t)t.width), py = (int)(idx / (size_t)t.width);
        const FaceRef fr = face_of(p.mesh, tag >> 4);
        const uint3 f = load_face(p.mesh, fr.face);
        CVFull a[kMaxClipVerts], b[kMaxClipVerts];
        a[0] = load_vertex<A>(p.mesh, f.x);
        a[1] = load_vertex<A>(p.mesh, f.y);
        a[2] = load_vertex<A>(p.mesh, f.z);
#pragma unroll
        for (int k = 0; k < 3; ++k) a[k].clip = mat4_mul(p.u.mvp, a[k].pos.x, a[k].pos.y, a[k].pos.z, 1.0f);
        CVFull* out;
        const int cnt = clip_triangle<A>(a, b, &out);
        const int j = (int)(tag & 7u);
        if (3 * j + 2 >= cnt) continue;  // cannot happen: the tag came from this clip
        Screen s;
        screen_setup(out[3 * j].clip, out[3 * j + 1].clip, out[3 * j + 2].clip, t.width, t.height, s);
        VSOut vo[3];
        for (int k = 0; k < 3; ++k) vo[k] = vertex_shader<S>(p.u, out[3 * j + k]);
        shade_winner<S>(p, idx, px, py, fr.material, s, vo);
    }
}

// Colour and/or depth fill, 16-byte stores (the planes are 256-byte aligned allocations).
__global__ void clear_kernel(uint32_t* color, float* depth, size_t n, uint32_t bgra, float dv, int do_color,
                             int do_depth) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t n4 = n / 4;
    const uint4 cv = make_uint4(bgra, bgra, bgra, bgra);
    const float4 dv4 = make_float4(dv, dv, dv, dv);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        if (do_color) reinterpret_cast<uint4*>(color)[i] = cv;
        if (do_depth) reinterpret_cast<float4*>(depth)[i] = dv4;
    }
    for (size_t i = 4 * n4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (do_color) color[i] = bgra;
        if (do_depth) depth[i] = dv;
    }
}

__global__ void fill_u64_kernel(unsigned long long* dst, size_t n, unsigned long long v) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = v;
}

__global__ void pack3_kernel(const float* __restrict__ src, float4* __restrict__ dst, uint32_t n) {
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = make_float4(src[3ull * i], src[3ull * i + 1], src[3ull * i + 2], 0.0f);
}

__device__ void debug_emit(float* out, uint32_t* count, uint32_t cap, const Screen& s, uint32_t tag) {
    if (is_backface(s)) return;
    uint32_t slot = atomicAdd(count, 1u);
    if (slot >= cap) return;
    float* o = out + 14ull * slot;
    o[0] = __uint_as_float(tag);
    for (int k = 0; k < 3; ++k) { o[1 + 2 * k] = s.x[k]; o[2 + 2 * k] = s.y[k]; o[7 + k] = s.z[k]; }
    o[10] = s.minx; o[11] = s.miny; o[12] = s.maxx; o[13] = s.maxy;
}

// Stage dump: the same clip / cull / setup as the geometry kernel, computed from the mesh
// directly (no vertex cache), writing one record per surviving triangle.
__global__ void debug_triangles_kernel(const __grid_constant__ DrawParams p, float* out, uint32_t* count,
                                       uint32_t cap) {
    uint32_t o = blockIdx.x * kBlock + threadIdx.x;
    if (o >= p.mesh.num_drawn || o > kMaxOrdinal) return;
    FaceRef fr = face_of(p.mesh, o);
    uint3 f = load_face(p.mesh, fr.face);
    const uint32_t nv = p.mesh.num_vertices;
    if (f.x >= nv || f.y >= nv || f.z >= nv) return;
    f4 c0 = load_clip(p.mesh, p.u.mvp, f.x), c1 = load_clip(p.mesh, p.u.mvp, f.y);
    f4 c2 = load_clip(p.mesh, p.u.mvp, f.z);
    int cls = clip_classify(c0, c1, c2);
    if (cls == 3) {
        Screen s;
        screen_setup(c0, c1, c2, p.target.width, p.target.height, s);
        debug_emit(out, count, cap, s, o << 4);
    } else if (cls < 0) {
        CVClip a[kMaxClipVerts], b[kMaxClipVerts];
        a[0].clip = c0; a[1].clip = c1; a[2].clip = c2;
        CVClip* res;
        int n = clip_triangle<0>(a, b, &res);
        for (int j = 0; 3 * j + 2 < n; ++j) {
            Screen s;
            screen_setup(res[3 * j].clip, res[3 * j + 1].clip, res[3 * j + 2].clip, p.target.width,
                         p.target.height, s);
            debug_emit(out, count, cap, s, (o << 4) | 8u | (uint32_t)j);
        }
    }
}

__global__ void debug_sample_kernel(DevTexture tex, const float2* uv, float4* out, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 q = uv[i];
    f4 c = tex_sample(tex, mk2(q.x, q.y));
    out[i] = make_float4(c.x, c.y, c.z, c.w);
}

unsigned grid_for(size_t n, int block, unsigned cap = 65535u * 16u) {
    size_t g = (n + (size_t)block - 1) / (size_t)block;
    if (g == 0) g = 1;
    return (unsigned)(g < cap ? g : cap);
}

template <int S>
cudaError_t launch_shaded(const DrawParams& p, const LaunchConfig& cfg, cudaStream_t stream, const AuxStream* aux,
                          cudaEvent_t* ev, uint64_t* launches) {
    cudaError_t e;
    auto mark = [&](int k) { return ev ? cudaEventRecord(ev[k], stream) : cudaSuccess; };
    if ((e = cudaMemsetAsync(p.scratch.counters, 0, kCountersReset, stream)) != cudaSuccess) return e;
    if ((e = mark(0)) != cudaSuccess) return e;
    if (p.mesh.num_drawn > 0) {
        vertex_kernel<S><<<grid_for(p.mesh.num_vertices, kBlock, 0x7FFFFFFFu), kBlock, 0, stream>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = mark(1)) != cudaSuccess) return e;
        geometry_kernel<<<grid_for(p.mesh.num_drawn, kBlock, 0x7FFFFFFFu), kBlock, 0, stream>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        *launches += 2;
    } else if ((e = mark(1)) != cudaSuccess) {
        return e;
    }
    if ((e = mark(2)) != cudaSuccess) return e;
    large_kernel<<<(unsigned)(cfg.num_sms * cfg.large_ctas_per_sm), kBlock, 0, stream>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = mark(3)) != cudaSuccess) return e;
    const unsigned tiles = (unsigned)(p.target.tiles_x * p.target.tiles_y);
    scan_kernel<<<min((tiles + 7u) / 8u, (unsigned)(cfg.num_sms * 8)), kBlock, 0, stream>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = mark(4)) != cudaSuccess) return e;
    // the clipped-winner pass is independent of the main shading pass: run it beside it
    cudaStream_t side = aux ? aux->stream : stream;
    if (aux) {
        if ((e = cudaEventRecord(aux->fork, stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(aux->stream, aux->fork, 0)) != cudaSuccess) return e;
    }
    resolve_clipped_kernel<S><<<(unsigned)cfg.num_sms / 2u + 1u, kBlock, 0, side>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    shade_kernel<S><<<(unsigned)(cfg.num_sms * cfg.resolve_ctas_per_sm), kBlock, 0, stream>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = mark(5)) != cudaSuccess) return e;
    if (aux) {
        if ((e = cudaEventRecord(aux->join, aux->stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(stream, aux->join, 0)) != cudaSuccess) return e;
    }
    *launches += 4;
    return mark(6);
}

}  // namespace

cudaError_t launch_draw(const DrawParams& p, const LaunchConfig& cfg, cudaStream_t stream, const AuxStream* aux,
                        cudaEvent_t* stage_events, uint64_t* launches) {
    switch (p.u.shader) {
        case kFlat: return launch_shaded<kFlat>(p, cfg, stream, aux, stage_events, launches);
        case kPhong: return launch_shaded<kPhong>(p, cfg, stream, aux, stage_events, launches);
        case kPBR: return launch_shaded<kPBR>(p, cfg, stream, aux, stage_events, launches);
        case kBlinnPhong: return launch_shaded<kBlinnPhong>(p, cfg, stream, aux, stage_events, launches);
        case kGouraud: return launch_shaded<kGouraud>(p, cfg, stream, aux, stage_events, launches);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_clear(uint32_t* color, float* depth, size_t pixels, uint32_t bgra, float depth_value,
                         bool do_color, bool do_depth, cudaStream_t stream) {
    clear_kernel<<<grid_for(pixels, 256, 4096), 256, 0, stream>>>(color, depth, pixels, bgra, depth_value,
                                                                  do_color ? 1 : 0, do_depth ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_fill_u64(unsigned long long* dst, size_t n, unsigned long long v, cudaStream_t stream) {
    fill_u64_kernel<<<grid_for(n, 256, 4096), 256, 0, stream>>>(dst, n, v);
    return cudaGetLastError();
}

cudaError_t launch_pack3(const float* src, float4* dst, uint32_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    pack3_kernel<<<grid_for(n, 256, 4096), 256, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_debug_triangles(const DrawParams& p, float* out, uint32_t* count, uint32_t capacity,
                                   cudaStream_t stream) {
    if (p.mesh.num_drawn == 0) return cudaSuccess;
    debug_triangles_kernel<<<grid_for(p.mesh.num_drawn, kBlock, 0x7FFFFFFFu), kBlock, 0, stream>>>(p, out, count,
                                                                                                   capacity);
    return cudaGetLastError();
}

cudaError_t launch_debug_sample(DevTexture tex, const float2* uv, float4* out, uint32_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    debug_sample_kernel<<<grid_for(n, 256, 0x7FFFFFFFu), 256, 0, stream>>>(tex, uv, out, n);
    return cudaGetLastError();
}

}  // namespace axr
