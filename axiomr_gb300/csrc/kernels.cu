// Draw kernels for sm_103a.
//
// A draw is three launches on one stream:
//   geometry_kernel  one thread per face in draw order: vertex transform (mvp * pos),
//                    homogeneous clipping, backface cull and triangle setup exactly as
//                    the reference (src/tiled_pipeline.cpp:195-236). Triangles whose
//                    pixel box is small are rasterised by the same thread; larger ones
//                    are appended (warp-aggregated atomics) to a list of LargeTri.
//   large_kernel     persistent warps take (large triangle, 16x16 tile) work items from
//                    a ragged queue: an entry cursor plus a per-entry tile counter.
//   resolve_kernel   persistent CTAs take dirty 16x16 tiles from the tile queue, one
//                    thread per pixel: the pixel's winning triangle is re-derived from
//                    its depth key, shaded once, and merged into the framebuffer with
//                    the reference's strict less-than depth test.
// Visibility is order independent: each covered pixel does a 64-bit atomicMin of
// (depth, draw-order position), so the surviving key is the reference's early-Z winner
// (minimum depth, earliest triangle on ties) whatever order the threads run in. Only
// the winning fragment is shaded; the reference shades every fragment that passes the
// early test at the time, with the same final colour.
#include <cuda_runtime.h>

#include "kernels.h"
#include "raster.cuh"
#include "shade.cuh"

namespace axr {

namespace {

constexpr int kBlock = 256;
constexpr uint32_t kTileFlagSet = 1u;

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

__device__ __forceinline__ void mark_tile(const DevTarget& t, DevCounters* c, int px, int py) {
    uint32_t tile = (uint32_t)(py >> 4) * (uint32_t)t.tiles_x + (uint32_t)(px >> 4);
    if (*reinterpret_cast<volatile uint32_t*>(&t.tile_flag[tile]) == 0u &&
        atomicExch(&t.tile_flag[tile], kTileFlagSet) == 0u) {
        uint32_t q = atomicAdd(&c->queue_len, 1u);
        t.tile_queue[q] = tile;  // at most one entry per tile: q < tiles_x * tiles_y
    }
}

// Visibility write of one covered pixel.
__device__ __forceinline__ void write_key(const DevTarget& t, DevCounters* c, int px, int py, float z, uint32_t tag) {
    if (!(z < __int_as_float(0x7f800000))) return;  // +inf and NaN never pass early-Z
    unsigned long long key = make_key(z, tag);
    unsigned long long* k = &t.key[(size_t)py * (size_t)t.width + (size_t)px];
    if (key < ld_relaxed(k)) {
        unsigned long long old = atomicMin(k, key);
        if (old > key && old == kEmptyKey) mark_tile(t, c, px, py);
    }
}

__device__ uint32_t raster_box(const DevTarget& t, DevCounters* c, const Edges& e, uint32_t tag) {
    uint32_t frags = 0;
    for (int py = e.y_lo; py < e.y_hi; ++py)
        for (int px = e.x_lo; px < e.x_hi; ++px) {
            PixelEval r = eval_pixel(e, px, py);
            if (r.covered) {
                ++frags;
                write_key(t, c, px, py, r.z, tag);
            }
        }
    return frags;
}

struct GeomStats {
    uint32_t tris, frags, large;
};

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

__device__ __forceinline__ uint32_t tiles_of(const Edges& e, uint32_t& ntx) {
    int tx0 = e.x_lo >> 4, tx1 = (e.x_hi - 1) >> 4;
    int ty0 = e.y_lo >> 4, ty1 = (e.y_hi - 1) >> 4;
    ntx = (uint32_t)(tx1 - tx0 + 1);
    return ntx * (uint32_t)(ty1 - ty0 + 1);
}

// Setup of one triangle that survived clipping; rasterises it or queues it as large.
__device__ void emit_triangle(const DrawParams& p, const Screen& s, uint32_t tag, GeomStats& st) {
    if (is_backface(s)) return;
    ++st.tris;
    Edges e;
    if (!edge_setup(s, p.target.width, p.target.height, e)) return;
    int npx = (e.x_hi - e.x_lo) * (e.y_hi - e.y_lo);
    DevCounters* c = p.scratch.counters;
    if (npx <= p.small_max_pixels) {
        st.frags += raster_box(p.target, c, e, tag);
        return;
    }
    // Large triangle: one setup record plus one work item per 16x16 tile of its box.
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
        // lists full: mark any reserved items as empty and rasterise here
        for (uint32_t k = base; k < icap && k - base < nt; ++k) p.scratch.items[k] = LargeItem{kNoItem, 0u};
        st.frags += raster_box(p.target, c, e, tag);
    }
}

__global__ void __launch_bounds__(kBlock) geometry_kernel(const __grid_constant__ DrawParams p) {
    GeomStats st = {0, 0, 0};
    uint32_t o = blockIdx.x * kBlock + threadIdx.x;
    if (o < p.mesh.num_drawn) {
        if (o > kMaxOrdinal) {
            atomicOr(&p.scratch.counters->error, kErrOrdinal);
        } else {
            FaceRef fr = face_of(p.mesh, o);
            uint3 f = load_face(p.mesh, fr.face);
            const uint32_t nv = p.mesh.num_vertices;
            int cls = 0;
            f4 c0, c1, c2;
            if (f.x >= nv || f.y >= nv || f.z >= nv) {
                atomicOr(&p.scratch.counters->error, kErrIndex);
            } else {
                c0 = load_clip(p.mesh, p.u.mvp, f.x);
                c1 = load_clip(p.mesh, p.u.mvp, f.y);
                c2 = load_clip(p.mesh, p.u.mvp, f.z);
                cls = clip_classify(c0, c1, c2);
            }
            if (cls == 3) {
                Screen s;
                screen_setup(c0, c1, c2, p.target.width, p.target.height, s);
                emit_triangle(p, s, o << 4, st);
            } else if (cls < 0) {
                CVClip a[kMaxClipVerts], b[kMaxClipVerts];
                a[0].clip = c0; a[1].clip = c1; a[2].clip = c2;
                CVClip* out;
                int n = clip_triangle<0>(a, b, &out);
                for (int j = 0; 3 * j + 2 < n; ++j) {
                    Screen s;
                    screen_setup(out[3 * j].clip, out[3 * j + 1].clip, out[3 * j + 2].clip, p.target.width,
                                 p.target.height, s);
                    emit_triangle(p, s, (o << 4) | 8u | (uint32_t)j, st);
                }
            }
        }
    }
    if (p.scratch.collect_stats) {
        unsigned full = 0xFFFFFFFFu;
        uint32_t t = __reduce_add_sync(full, st.tris), f = __reduce_add_sync(full, st.frags);
        uint32_t l = __reduce_add_sync(full, st.large);
        if ((threadIdx.x & 31) == 0) {
            DevCounters* c = p.scratch.counters;
            if (t) atomicAdd(&c->stat_triangles, (unsigned long long)t);
            if (f) atomicAdd(&c->stat_fragments, (unsigned long long)f);
            if (l) atomicAdd(&c->stat_large, (unsigned long long)l);
        }
    }
}

// Last CTA out resets the counters this kernel consumed.
__device__ __forceinline__ bool last_cta(uint32_t* done_counter) {
    __shared__ uint32_t s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = (atomicAdd(done_counter, 1u) == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    return s_last != 0u;
}

__global__ void __launch_bounds__(kBlock) large_kernel(const __grid_constant__ DrawParams p) {
    DevCounters* c = p.scratch.counters;
    const uint32_t n_items = min(*reinterpret_cast<volatile uint32_t*>(&c->item_count), p.scratch.item_cap);
    const uint32_t n_tris = min(*reinterpret_cast<volatile uint32_t*>(&c->large_count), p.scratch.large_cap);
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
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int py = ty * kTile + (lane >> 4) + 2 * r;
                if (px >= e.x_lo && px < e.x_hi && py >= e.y_lo && py < e.y_hi) {
                    PixelEval pe = eval_pixel(e, px, py);
                    if (pe.covered) {
                        ++frags;
                        write_key(p.target, c, px, py, pe.z, tag);
                    }
                }
            }
        }
    }
    if (p.scratch.collect_stats) {
        uint32_t f = __reduce_add_sync(0xFFFFFFFFu, frags);
        if (lane == 0 && f) atomicAdd(&c->stat_fragments, (unsigned long long)f);
    }
    if (last_cta(&c->large_done) && threadIdx.x == 0) {
        c->large_count = 0u;
        c->item_count = 0u;
        c->item_head = 0u;
        c->large_done = 0u;
    }
}

// Re-derive the winning triangle of a pixel from its key tag and shade it.
template <int S>
__device__ void resolve_pixel(const DrawParams& p, int px, int py) {
    const DevTarget& t = p.target;
    size_t idx = (size_t)py * (size_t)t.width + (size_t)px;
    unsigned long long key = t.key[idx];
    if (key == kEmptyKey) return;
    t.key[idx] = kEmptyKey;
    const uint32_t tag = (uint32_t)key;
    constexpr int A = ShaderAttrs<S>::mask;
    FaceRef fr = face_of(p.mesh, tag >> 4);
    uint3 f = load_face(p.mesh, fr.face);
    CVFull v[3];
    v[0] = load_vertex<A>(p.mesh, f.x);
    v[1] = load_vertex<A>(p.mesh, f.y);
    v[2] = load_vertex<A>(p.mesh, f.z);
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k].clip = mat4_mul(p.u.mvp, v[k].pos.x, v[k].pos.y, v[k].pos.z, 1.0f);
    if (tag & 8u) {
        CVFull a[kMaxClipVerts], b[kMaxClipVerts];
        a[0] = v[0]; a[1] = v[1]; a[2] = v[2];
        CVFull* out;
        int n = clip_triangle<A>(a, b, &out);
        int j = (int)(tag & 7u);
        if (3 * j + 2 >= n) return;  // cannot happen: the tag came from this clip
        v[0] = out[3 * j]; v[1] = out[3 * j + 1]; v[2] = out[3 * j + 2];
    }
    Screen s;
    screen_setup(v[0].clip, v[1].clip, v[2].clip, t.width, t.height, s);
    Edges e;
    if (!edge_setup(s, t.width, t.height, e)) return;
    PixelEval r = eval_pixel(e, px, py);
    if (!(r.z < t.depth[idx])) return;  // merge: tile depth < framebuffer depth (strict)
    VSOut vo[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) vo[k] = vertex_shader<S>(p.u, v[k]);
    f4 col = fragment_shader<S>(p.u, p.mesh.materials[fr.material], mk3(r.alpha, r.beta, r.gamma), vo);
    t.color[idx] = pack_bgra(col);
    t.depth[idx] = r.z;
}

// One CTA per possible queue slot (the grid covers every tile of the target); CTAs past
// the number of dirty tiles exit at once, so all dirty tiles are resolved concurrently.
template <int S>
__global__ void __launch_bounds__(kBlock) resolve_kernel(const __grid_constant__ DrawParams p) {
    DevCounters* c = p.scratch.counters;
    const DevTarget& t = p.target;
    const uint32_t qlen = *reinterpret_cast<volatile uint32_t*>(&c->queue_len);
    if (blockIdx.x < qlen) {
        const uint32_t tile = t.tile_queue[blockIdx.x];
        const int px = (int)(tile % (uint32_t)t.tiles_x) * kTile + (threadIdx.x & 15);
        const int py = (int)(tile / (uint32_t)t.tiles_x) * kTile + (threadIdx.x >> 4);
        if (px < t.width && py < t.height) resolve_pixel<S>(p, px, py);
        if (threadIdx.x == 0) {
            t.tile_flag[tile] = 0u;
            if (p.scratch.collect_stats) atomicAdd(&c->stat_tiles, 1ull);
        }
    }
    if (last_cta(&c->resolve_done) && threadIdx.x == 0) {
        c->queue_len = 0u;
        c->queue_head = 0u;
        c->resolve_done = 0u;
    }
}

__global__ void clear_kernel(uint32_t* color, float* depth, size_t n, uint32_t bgra, float dv, int do_color,
                             int do_depth) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
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
cudaError_t launch_resolve(const DrawParams& p, unsigned grid, cudaStream_t stream) {
    resolve_kernel<S><<<grid, kBlock, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_draw(const DrawParams& p, const LaunchConfig& cfg, cudaStream_t stream,
                        cudaEvent_t* stage_events, uint64_t* launches) {
    cudaError_t e;
    if (stage_events && (e = cudaEventRecord(stage_events[0], stream)) != cudaSuccess) return e;
    if (p.mesh.num_drawn > 0) {
        geometry_kernel<<<grid_for(p.mesh.num_drawn, kBlock, 0x7FFFFFFFu), kBlock, 0, stream>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        ++*launches;
    }
    if (stage_events && (e = cudaEventRecord(stage_events[1], stream)) != cudaSuccess) return e;
    unsigned lg = (unsigned)(cfg.num_sms * cfg.large_ctas_per_sm);
    large_kernel<<<lg > 0 ? lg : 1, kBlock, 0, stream>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ++*launches;
    if (stage_events && (e = cudaEventRecord(stage_events[2], stream)) != cudaSuccess) return e;
    unsigned rg = (unsigned)(p.target.tiles_x * p.target.tiles_y);
    switch (p.u.shader) {
        case kFlat: e = launch_resolve<kFlat>(p, rg, stream); break;
        case kPhong: e = launch_resolve<kPhong>(p, rg, stream); break;
        case kPBR: e = launch_resolve<kPBR>(p, rg, stream); break;
        case kBlinnPhong: e = launch_resolve<kBlinnPhong>(p, rg, stream); break;
        case kGouraud: e = launch_resolve<kGouraud>(p, rg, stream); break;
        default: e = cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    ++*launches;
    if (stage_events) return cudaEventRecord(stage_events[3], stream);
    return cudaSuccess;
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
