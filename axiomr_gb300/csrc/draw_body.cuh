// Device-side steps of one draw, shared by the per-draw kernels (kernels.cu) and the
// batched persistent kernel (batch.cu): per-vertex transform and shading, per-face clip /
// cull / setup / small-triangle raster, the large-triangle tile raster, and the shading of
// one pixel's winning fragment. The kernels differ only in how work is handed out.
#pragma once
#include <cuda_runtime.h>

#include "raster.cuh"
#include "shade.cuh"

namespace axr {
namespace {

constexpr uint32_t kNoTile = 0xFFFFFFFFu;

// Tag bit of an unclipped triangle that left a shading record (clipped triangles use bits
// 0-3 for 8 + their clip index; an unclipped one has them free). Both shading paths give
// the same bits; the record saves re-deriving the setup, which pays off when the
// triangle's box holds at least kRecMinPixels pixels.
constexpr uint32_t kRecTag = 1u;
constexpr int kRecMinPixels = 16;

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
    uint32_t tris, frags, large, tested;
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
            st.tested += (uint32_t)(ex - sx);
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

// Raster record (kRasterRec float4, see device_types.h): edges, 1/area, depths, pixel range
// and one extra word (material or tag).
__device__ __forceinline__ void store_raster(float4* r, const Edges& e, uint32_t word) {
    r[0] = make_float4(e.a[0], e.b[0], e.c[0], e.a[1]);
    r[1] = make_float4(e.b[1], e.c[1], e.a[2], e.b[2]);
    r[2] = make_float4(e.c[2], e.inv_area, e.z[0], e.z[1]);
    const uint32_t xs = (uint32_t)e.x_lo | ((uint32_t)e.x_hi << 16);
    const uint32_t ys = (uint32_t)e.y_lo | ((uint32_t)e.y_hi << 16);
    r[3] = make_float4(e.z[2], __uint_as_float(xs), __uint_as_float(ys), __uint_as_float(word));
}

__device__ __forceinline__ uint32_t unpack_raster(const float4 r0, const float4 r1, const float4 r2, const float4 r3,
                                                  Edges& e) {
    e.a[0] = r0.x; e.b[0] = r0.y; e.c[0] = r0.z; e.a[1] = r0.w;
    e.b[1] = r1.x; e.c[1] = r1.y; e.a[2] = r1.z; e.b[2] = r1.w;
    e.c[2] = r2.x; e.inv_area = r2.y; e.z[0] = r2.z; e.z[1] = r2.w;
    e.z[2] = r3.x;
    const uint32_t xs = __float_as_uint(r3.y), ys = __float_as_uint(r3.z);
    e.x_lo = (int)(xs & 0xFFFFu); e.x_hi = (int)(xs >> 16);
    e.y_lo = (int)(ys & 0xFFFFu); e.y_hi = (int)(ys >> 16);
    return __float_as_uint(r3.w);
}

__device__ __forceinline__ void store_record(const DrawParams& p, uint32_t ordinal, const Edges& e, uint32_t material,
                                             const uint3& f) {
    float4* r = p.scratch.rec + (size_t)kRecFloat4 * ordinal;
    store_raster(r, e, material);
    r[4] = make_float4(__uint_as_float(f.x), __uint_as_float(f.y), __uint_as_float(f.z), 0.0f);
}

// kCoherent: the record was written earlier in the same launch (plain loads).
template <bool kCoherent>
__device__ __forceinline__ uint32_t load_record(const DrawParams& p, uint32_t ordinal, Edges& e, uint3& f) {
    const float4* r = p.scratch.rec + (size_t)kRecFloat4 * ordinal;
    const float4 r0 = ld_cached<kCoherent>(r), r1 = ld_cached<kCoherent>(r + 1), r2 = ld_cached<kCoherent>(r + 2);
    const float4 r3 = ld_cached<kCoherent>(r + 3), r4 = ld_cached<kCoherent>(r + 4);
    const uint32_t material = unpack_raster(r0, r1, r2, r3, e);
    f = make_uint3(__float_as_uint(r4.x), __float_as_uint(r4.y), __float_as_uint(r4.z));
    return material;
}

// One triangle that survived clipping: cull, set up, then rasterise it here or queue its
// tiles. *single_tile receives the one tile a small triangle wrote to (the caller marks
// it after deduplicating across the warp); boxes spanning several tiles are marked here.
// An unclipped triangle that can win a pixel leaves its shading record (face f, material).
__device__ void emit_triangle(const DrawParams& p, const Screen& s, uint32_t tag, GeomStats& st,
                              uint32_t* single_tile, const uint3& f, uint32_t material) {
    if (is_backface(s)) return;
    ++st.tris;
    Edges e;
    if (!edge_setup(s, p.target.width, p.target.height, e)) return;
    const int npx = (e.x_hi - e.x_lo) * (e.y_hi - e.y_lo);
    const bool record = (tag & 8u) == 0u && npx >= kRecMinPixels;
    if (record) tag |= kRecTag;
    DevCounters* c = p.scratch.counters;
    if (npx <= p.small_max_pixels) {
        if (raster_box(p.target, e, tag, st)) {
            if (record) store_record(p, tag >> 4, e, material, f);
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
    if (record) store_record(p, tag >> 4, e, material, f);
    if (slot < p.scratch.large_cap && base + nt <= icap && base + nt > base) {
        store_large(&p.scratch.large[slot], e, tag);
        if (p.scratch.large_draw) p.scratch.large_draw[slot] = p.draw;
        for (uint32_t k = 0; k < nt; ++k) p.scratch.items[base + k] = LargeItem{slot, k};
        ++st.large;
    } else {
        // lists full: mark the reserved items empty and rasterise the triangle here
        for (uint32_t k = base; k < icap && k - base < nt; ++k) p.scratch.items[k] = LargeItem{kNoItem, 0u};
        if (raster_box(p.target, e, tag, st)) mark_box(p.target, e);
    }
}


// IShader::vertex of vertex i plus its screen position, NDC depth and clip-plane masks
// (the per-vertex part of the reference's Triangle ctor, src/tiled_pipeline.cpp:53-72).
template <int S>
__device__ __forceinline__ void vertex_one(const DrawParams& p, uint32_t i) {
    constexpr int A = ShaderAttrs<S>::mask;
    CVFull v = load_vertex<A>(p.mesh, i);
    f4 clip = mat4_mul(p.u.mvp, v.pos.x, v.pos.y, v.pos.z, 1.0f);
    f3 sc = screen_vertex(clip, (float)p.target.width, (float)p.target.height);
    p.scratch.vscreen[i] = make_float4(sc.x, sc.y, sc.z, __uint_as_float(plane_masks(clip)));
    pack_vsout<S>(vertex_shader<S>(p.u, v), &p.scratch.vattr[(size_t)VAttr<S>::n * i]);
}

// A face whose vertices straddle the clip volume: the clipper's output triangles, each
// emitted with its clip index in the tag and its tile marked here.
__device__ __noinline__ void geometry_clipped(const DrawParams& p, uint32_t o, const uint3 f, uint32_t material,
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
        uint32_t tile = kNoTile;
        emit_triangle(p, s, (o << 4) | 8u | (uint32_t)j, st, &tile, f, material);
        if (tile != kNoTile) mark_tile(p.target, tile);
    }
}

// Face at draw-order position o (< num_drawn): clip classification, cull, setup and
// raster or queueing (src/tiled_pipeline.cpp:195-240, 436-487).
// kCoherent: the vertex cache was written earlier in the same launch (plain loads).
template <bool kCoherent = false>
__device__ __forceinline__ void geometry_one(const DrawParams& p, uint32_t o, GeomStats& st, uint32_t& single_tile) {
    if (o > kMaxOrdinal) {
        atomicOr(&p.scratch.counters->error, kErrOrdinal);
        return;
    }
    const FaceRef fr = face_of(p.mesh, o);
    const uint3 f = load_face(p.mesh, fr.face);
    const uint32_t nv = p.mesh.num_vertices;
    if (f.x >= nv || f.y >= nv || f.z >= nv) {
        atomicOr(&p.scratch.counters->error, kErrIndex);
        return;
    }
    const float4* vs = p.scratch.vscreen;
    const float4 g0 = ld_cached<kCoherent>(&vs[f.x]), g1 = ld_cached<kCoherent>(&vs[f.y]),
                 g2 = ld_cached<kCoherent>(&vs[f.z]);
    const int cls = classify_masks(__float_as_uint(g0.w), __float_as_uint(g1.w), __float_as_uint(g2.w));
    if (cls == 3) {
        Screen s;
        s.x[0] = g0.x; s.y[0] = g0.y; s.z[0] = g0.z;
        s.x[1] = g1.x; s.y[1] = g1.y; s.z[1] = g1.z;
        s.x[2] = g2.x; s.y[2] = g2.y; s.z[2] = g2.z;
        screen_bbox(s);
        emit_triangle(p, s, o << 4, st, &single_tile, f, fr.material);
    } else if (cls < 0) {
        geometry_clipped(p, o, f, fr.material, st);
    }
}

// A front-facing face inside the clip volume, queued by geometry_front for the setup and
// raster pass of the compacted face phase.
struct FaceJob {
    float x[3], y[3], z[3];
    uint32_t o, material;
    uint32_t f[3];
};

// The first half of geometry_one for the compacted face phase: the checks, the vertex-cache
// gathers, clip classification and the back-face test. A face that straddles the clip
// volume is finished here; one inside it that faces the camera is returned in *job (true)
// for emit_triangle in a second pass, where every lane of a warp has such a face.
template <bool kCoherent>
__device__ __forceinline__ bool geometry_front(const DrawParams& p, uint32_t o, GeomStats& st, FaceJob& job) {
    if (o > kMaxOrdinal) {
        atomicOr(&p.scratch.counters->error, kErrOrdinal);
        return false;
    }
    const FaceRef fr = face_of(p.mesh, o);
    const uint3 f = load_face(p.mesh, fr.face);
    const uint32_t nv = p.mesh.num_vertices;
    if (f.x >= nv || f.y >= nv || f.z >= nv) {
        atomicOr(&p.scratch.counters->error, kErrIndex);
        return false;
    }
    const float4* vs = p.scratch.vscreen;
    const float4 g0 = ld_cached<kCoherent>(&vs[f.x]), g1 = ld_cached<kCoherent>(&vs[f.y]),
                 g2 = ld_cached<kCoherent>(&vs[f.z]);
    const int cls = classify_masks(__float_as_uint(g0.w), __float_as_uint(g1.w), __float_as_uint(g2.w));
    if (cls == 3) {
        Screen s;
        s.x[0] = g0.x; s.y[0] = g0.y; s.z[0] = g0.z;
        s.x[1] = g1.x; s.y[1] = g1.y; s.z[1] = g1.z;
        s.x[2] = g2.x; s.y[2] = g2.y; s.z[2] = g2.z;
        if (is_backface(s)) return false;
        job = FaceJob{{s.x[0], s.x[1], s.x[2]}, {s.y[0], s.y[1], s.y[2]}, {s.z[0], s.z[1], s.z[2]},
                      o, fr.material, {f.x, f.y, f.z}};
        return true;
    }
    if (cls < 0) geometry_clipped(p, o, f, fr.material, st);
    return false;
}

// The second half: setup and raster (or queueing) of a queued face, as geometry_one does.
__device__ __forceinline__ void geometry_job(const DrawParams& p, const FaceJob& j, GeomStats& st,
                                             uint32_t& single_tile) {
    Screen s;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s.x[k] = j.x[k];
        s.y[k] = j.y[k];
        s.z[k] = j.z[k];
    }
    screen_bbox(s);
    emit_triangle(p, s, j.o << 4, st, &single_tile, make_uint3(j.f[0], j.f[1], j.f[2]), j.material);
}

// Warp-wide end of the geometry step: one mark per distinct single tile in the warp, and
// the statistics. All 32 lanes must call it.
__device__ __forceinline__ void geometry_warp_tail(const DevTarget& t, DevCounters* c, bool stats, const GeomStats& st,
                                                   uint32_t single_tile) {
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, single_tile);
    if (single_tile != kNoTile && (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) mark_tile(t, single_tile);
    if (stats) {
        const unsigned full = 0xFFFFFFFFu;
        uint32_t tr = __reduce_add_sync(full, st.tris), fr = __reduce_add_sync(full, st.frags);
        uint32_t l = __reduce_add_sync(full, st.large), te = __reduce_add_sync(full, st.tested);
        if ((threadIdx.x & 31) == 0) {
            if (tr) atomicAdd(&c->stat_triangles, (unsigned long long)tr);
            if (fr) atomicAdd(&c->stat_fragments, (unsigned long long)fr);
            if (l) atomicAdd(&c->stat_large, (unsigned long long)l);
            if (te) atomicAdd(&c->stat_tested, (unsigned long long)te);
        }
    }
}

// One CTA's faces in two passes (every thread calls it with its face o; *count is zero on
// entry; `jobs` holds one entry per thread): geometry_front per face, then geometry_job on
// the front-facing faces inside the clip volume. When fewer than three quarters of the
// CTA's faces go on (a closed mesh turns about half of its faces away), they are first
// compacted into `jobs` by warp ballots, so that the second pass runs with every lane
// busy instead of idling the culled faces' lanes through their neighbours' raster loops;
// otherwise each thread goes on with its own face (the shared-memory round trip would
// cost more than the idle lanes).
__device__ __forceinline__ void geometry_compacted(const DrawParams& p, uint32_t o, DevCounters* c, bool stats,
                                                   FaceJob* jobs, uint32_t* count) {
    GeomStats st = {0, 0, 0, 0};
    uint32_t single_tile = kNoTile;
    FaceJob job;
    const bool queued = o < p.mesh.num_drawn && geometry_front<false>(p, o, st, job);
    const unsigned m = __ballot_sync(0xFFFFFFFFu, queued);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0 && m) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    __syncthreads();
    const uint32_t n = *count;
    if (4u * n >= 3u * blockDim.x) {
        if (queued) geometry_job(p, job, st, single_tile);
    } else {
        if (queued) jobs[base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = job;
        __syncthreads();
        if (threadIdx.x < n) geometry_job(p, jobs[threadIdx.x], st, single_tile);
    }
    geometry_warp_tail(p.target, c, stats, st, single_tile);
}

// Whether no pixel of 16x16 tile (tx, ty) inside the triangle's box can test covered.
// Each edge function is linear, so over the tile's pixel centres it peaks at a corner of
// their rectangle. eval_pixel's float evaluation of an edge at a centre is within a few
// units of 2^-24 * M of its exact value, M = |a|(|x|+16) + |b||y| + |c| bounding the
// magnitudes of its terms, and the corner values here are within 3 such units; if the
// corner maximum of some edge is below -64 * 2^-24 * M, every evaluated value of that edge
// in the tile is negative, so the tile holds no covered pixel and is skipped.
__device__ __forceinline__ bool tile_outside(const Edges& e, int tx, int ty) {
    const float x0 = (float)max(tx * kTile, e.x_lo) + 0.5f, x1 = (float)min(tx * kTile + kTile, e.x_hi) - 0.5f;
    const float y0 = (float)max(ty * kTile, e.y_lo) + 0.5f, y1 = (float)min(ty * kTile + kTile, e.y_hi) - 0.5f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = e.a[k], b = e.b[k], c = e.c[k];
        const float ex = a >= 0.f ? a * x1 : a * x0;  // the larger of a*x0, a*x1
        const float ey = b >= 0.f ? b * y1 : b * y0;
        const float emax = (ex + ey) + c;
        const float m = fabsf(a) * (fabsf(x1) + 16.0f) + fabsf(b) * fabsf(y1) + fabsf(c);
        if (emax < -64.0f * 5.9604645e-8f * m) return true;
    }
    return false;
}

// One large-triangle work item: the warp evaluates the 256 pixels of tile `item_tile` of
// the triangle's tile box, 8 per lane, and flags the tile if a key was written.
__device__ __forceinline__ void large_tile(const DevTarget& t, const Edges& e, uint32_t tag, uint32_t item_tile,
                                           uint32_t& frags, uint32_t& tested) {
    const int lane = threadIdx.x & 31;
    uint32_t ntx;
    tiles_of(e, ntx);
    const int tx = (e.x_lo >> 4) + (int)(item_tile % ntx);
    const int ty = (e.y_lo >> 4) + (int)(item_tile / ntx);
    if (tile_outside(e, tx, ty)) return;
    const int px = tx * kTile + (lane & 15);
    bool wrote = false;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int py = ty * kTile + (lane >> 4) + 2 * r;
        if (px >= e.x_lo && px < e.x_hi && py >= e.y_lo && py < e.y_hi) {
            ++tested;
            PixelEval pe = eval_pixel(e, px, py);
            if (pe.covered) {
                ++frags;
                wrote |= write_key(t, px, py, pe.z, tag);
            }
        }
    }
    if (__any_sync(0xFFFFFFFFu, wrote) && lane == 0) mark_tile(t, (uint32_t)ty * (uint32_t)t.tiles_x + (uint32_t)tx);
}

// Winner inputs of an unclipped tag without a record: screen positions from the vertex
// cache and the cached vertex-shader outputs.
template <int S, bool kCoherent = false>
__device__ __forceinline__ uint32_t winner_inputs(const DrawParams& p, uint32_t tag, Screen& s, VSOut* vo) {
    const FaceRef fr = face_of(p.mesh, tag >> 4);
    const uint3 f = load_face(p.mesh, fr.face);
    const uint32_t vi[3] = {f.x, f.y, f.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 g = ld_cached<kCoherent>(&p.scratch.vscreen[vi[k]]);
        s.x[k] = g.x;
        s.y[k] = g.y;
        s.z[k] = g.z;
        vo[k] = unpack_vsout<S, kCoherent>(&p.scratch.vattr[(size_t)VAttr<S>::n * vi[k]]);
    }
    screen_bbox(s);
    return fr.material;
}

// Winner inputs of an unclipped tag: its shading record and the cached vertex-shader
// outputs of its three vertices. Returns the material.
template <int S, bool kCoherent = false>
__device__ __forceinline__ uint32_t record_inputs(const DrawParams& p, uint32_t tag, Edges& e, VSOut* vo) {
    uint3 f;
    const uint32_t material = load_record<kCoherent>(p, tag >> 4, e, f);
    const uint32_t vi[3] = {f.x, f.y, f.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) vo[k] = unpack_vsout<S, kCoherent>(&p.scratch.vattr[(size_t)VAttr<S>::n * vi[k]]);
    return material;
}

// Winner inputs of a clipped tag: the clipper re-run on the face's raw vertex attributes
// (the geometry stage's clip, now carrying attributes; src/pipeline.cpp:243-272), output
// triangle j of the tag. Returns false if the tag names no output triangle.
template <int S>
__device__ bool clipped_inputs(const DrawParams& p, uint32_t tag, Screen& s, VSOut* vo, uint32_t& material) {
    constexpr int A = ShaderAttrs<S>::mask;
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
    if (3 * j + 2 >= cnt) return false;  // cannot happen: the tag came from this clip
    screen_setup(out[3 * j].clip, out[3 * j + 1].clip, out[3 * j + 2].clip, p.target.width, p.target.height, s);
    for (int k = 0; k < 3; ++k) vo[k] = vertex_shader<S>(p.u, out[3 * j + k]);
    material = fr.material;
    return true;
}

// Fragment of the winner at (px, py): exact barycentrics and depth, the merge test against
// `old_depth` (tile depth < framebuffer depth, strict; src/tiled_pipeline.cpp:1171-1174)
// and the shader. Returns whether the fragment is written.
template <int S>
__device__ __forceinline__ bool shade_pixel(const DrawParams& p, int px, int py, uint32_t material, Screen& s,
                                            const VSOut* vo, float old_depth, uint32_t& bgra, float& z) {
    Edges e;
    if (!edge_setup(s, p.target.width, p.target.height, e)) return false;
    const PixelEval r = eval_pixel(e, px, py);
    if (!(r.z < old_depth)) return false;
    const f4 col = fragment_shader<S>(p.u, p.mesh.materials[material], mk3(r.alpha, r.beta, r.gamma), vo);
    bgra = pack_bgra(col);
    z = r.z;
    return true;
}

}  // namespace
}  // namespace axr

namespace axr {
namespace {

// Fragment of the unclipped winner `tag` at (px, py): the setup from its shading record
// when it has one, else re-derived from the face; then exact barycentrics and depth, the
// strict merge test against `old_depth` and the shader. Returns whether it is written.
// Fragment at (px, py) of a triangle given its setup, vertex-shader outputs and material:
// exact barycentrics and depth, the strict merge test against `old_depth` and the shader.
template <int S>
__device__ __forceinline__ bool shade_from(const DrawParams& p, const Edges& e, const VSOut* vo, uint32_t material,
                                           int px, int py, float old_depth, uint32_t& bgra, float& z) {
    const PixelEval r = eval_pixel(e, px, py);
    if (!(r.z < old_depth)) return false;
    const f4 col = fragment_shader<S>(p.u, p.mesh.materials[material], mk3(r.alpha, r.beta, r.gamma), vo);
    bgra = pack_bgra(col);
    z = r.z;
    return true;
}

template <int S, bool kCoherent = false>
__device__ __forceinline__ bool shade_unclipped(const DrawParams& p, uint32_t tag, int px, int py, float old_depth,
                                                uint32_t& bgra, float& z) {
    VSOut vo[3];
    Edges e;
    uint32_t material;
    if (tag & kRecTag) {
        material = record_inputs<S, kCoherent>(p, tag, e, vo);
    } else {
        Screen s;
        material = winner_inputs<S, kCoherent>(p, tag, s, vo);
        if (!edge_setup(s, p.target.width, p.target.height, e)) return false;
    }
    return shade_from<S>(p, e, vo, material, px, py, old_depth, bgra, z);
}

// Winner that came out of the clipper: its inputs from the clipper re-run, then the
// fragment; kept out of line so that the clipper's state does not raise the register count
// of the shading loops that call it.
template <int S>
__device__ __noinline__ bool shade_clipped_px(const DrawParams& p, uint32_t tag, int px, int py, float old_depth,
                                              uint32_t* bgra, float* z) {
    Screen s;
    VSOut vo[3];
    uint32_t material;
    return clipped_inputs<S>(p, tag, s, vo, material) && shade_pixel<S>(p, px, py, material, s, vo, old_depth, *bgra, *z);
}

}  // namespace
}  // namespace axr
