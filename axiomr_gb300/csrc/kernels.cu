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
#include <cstring>

#include "draw_body.cuh"
#include "kernels.h"

namespace axr {

namespace {

constexpr int kBlock = 256;

// Resident 256-thread CTAs per SM the geometry kernel is compiled for (register budget
// 65536 / (256 * n)); 5 keeps it at 48 registers.
#ifndef AXR_GEOMETRY_MIN_BLOCKS
#define AXR_GEOMETRY_MIN_BLOCKS 5
#endif

template <int S>
__global__ void __launch_bounds__(kBlock) vertex_kernel(const __grid_constant__ DrawParams p) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < p.mesh.num_vertices) vertex_one<S>(p, i);
}

__global__ void __launch_bounds__(kBlock, AXR_GEOMETRY_MIN_BLOCKS) geometry_kernel(const __grid_constant__ DrawParams p) {
    GeomStats st = {0, 0, 0, 0};
    uint32_t single_tile = kNoTile;
    const uint32_t o = blockIdx.x * kBlock + threadIdx.x;
    if (o < p.mesh.num_drawn) geometry_one(p, o, st, single_tile);
    geometry_warp_tail(p.target, p.scratch.counters, p.scratch.collect_stats != 0, st, single_tile);
}

__global__ void __launch_bounds__(kBlock) large_kernel(const __grid_constant__ DrawParams p) {
    DevCounters* c = p.scratch.counters;
    const uint32_t n_items = min(ld_volatile(&c->item_count), p.scratch.item_cap);
    if (n_items == 0) return;
    const uint32_t n_tris = min(ld_volatile(&c->large_count), p.scratch.large_cap);
    const int lane = threadIdx.x & 31;
    uint32_t frags = 0, tested = 0;
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
            large_tile(p.target, e, tag, item.tile, frags, tested);
        }
    }
    if (p.scratch.collect_stats) {
        uint32_t f = __reduce_add_sync(0xFFFFFFFFu, frags);
        const uint32_t te = __reduce_add_sync(0xFFFFFFFFu, tested);
        if (lane == 0 && f) atomicAdd(&c->stat_fragments, (unsigned long long)f);
        if (lane == 0 && te) atomicAdd(&c->stat_tested, (unsigned long long)te);
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
                if (p.scratch.collect_stats) {
                    atomicAdd(&c->stat_tiles, 1ull);
                    atomicAdd(&c->stat_shaded, (unsigned long long)(ns + nc));
                }
            }
        }
        __syncthreads();
    }
}

// Dense shading of the covered pixels whose winner is unclipped: the winner's setup (from
// its shading record, or re-derived from the face and the vertex cache) gives its exact
// barycentrics and depth, and the fragment is shaded once.
template <int S>
__global__ void __launch_bounds__(kBlock) shade_kernel(const __grid_constant__ DrawParams p) {
    DevCounters* c = p.scratch.counters;
    const DevTarget& t = p.target;
    const uint32_t n = min(ld_volatile(&c->shade_count), p.scratch.px_cap);
    for (uint32_t q = blockIdx.x * kBlock + threadIdx.x; q < n; q += gridDim.x * kBlock) {
        const uint2 w = p.scratch.shade[q];
        const size_t idx = w.x;
        const int px = (int)(idx % (size_t)t.width), py = (int)(idx / (size_t)t.width);
        uint32_t bgra;
        float z;
        if (shade_unclipped<S>(p, w.y, px, py, t.depth[idx], bgra, z)) {
            t.color[idx] = bgra;
            t.depth[idx] = z;
        }
    }
}

// Pixels whose winner is a clipped triangle: the winner's inputs come from re-running the
// clipper on the face.
template <int S>
__global__ void __launch_bounds__(kBlock) resolve_clipped_kernel(const __grid_constant__ DrawParams p) {
    const uint32_t n = min(ld_volatile(&p.scratch.counters->clip_count), p.scratch.px_cap);
    const DevTarget& t = p.target;
    for (uint32_t q = blockIdx.x * kBlock + threadIdx.x; q < n; q += gridDim.x * kBlock) {
        const uint2 w = p.scratch.clip_px[q];
        const size_t idx = w.x;
        const int px = (int)(idx % (size_t)t.width), py = (int)(idx / (size_t)t.width);
        Screen s;
        VSOut vo[3];
        uint32_t material;
        if (!clipped_inputs<S>(p, w.y, s, vo, material)) continue;
        uint32_t bgra;
        float z;
        if (shade_pixel<S>(p, px, py, material, s, vo, t.depth[idx], bgra, z)) {
            t.color[idx] = bgra;
            t.depth[idx] = z;
        }
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
    // (unless no triangle can have been clipped, when its list is empty)
    const bool clipped = !cfg.clip_free;
    cudaStream_t side = aux ? aux->stream : stream;
    if (clipped && aux) {
        if ((e = cudaEventRecord(aux->fork, stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(aux->stream, aux->fork, 0)) != cudaSuccess) return e;
    }
    if (clipped) {
        resolve_clipped_kernel<S><<<(unsigned)cfg.num_sms / 2u + 1u, kBlock, 0, side>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    shade_kernel<S><<<(unsigned)(cfg.num_sms * cfg.resolve_ctas_per_sm), kBlock, 0, stream>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = mark(5)) != cudaSuccess) return e;
    if (clipped && aux) {
        if ((e = cudaEventRecord(aux->join, aux->stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(stream, aux->join, 0)) != cudaSuccess) return e;
    }
    *launches += clipped ? 4 : 3;
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

// ---- mesh bounds after an update (batch planning's density classes)
__device__ __forceinline__ uint32_t float_ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_float(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

__global__ void mesh_box_kernel(const float4* __restrict__ pos, uint32_t n, MeshBounds* out) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = __ldg(pos + i);
        const float v[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], v[k]);
            hi[k] = fmaxf(hi[k], v[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&out->lo[k], float_ord(lo[k]));
            atomicMax(&out->hi[k], float_ord(hi[k]));
        }
    }
}

__global__ void mesh_radius_kernel(const float4* __restrict__ pos, uint32_t n, MeshBounds* out) {
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = __fmul_rn(0.5f, __fadd_rn(ord_float(out->lo[k]), ord_float(out->hi[k])));
    double r2 = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = __ldg(pos + i);
        const float v[3] = {p.x, p.y, p.z};
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double t = __dsub_rn((double)v[k], (double)c[k]);
            s = __dadd_rn(s, __dmul_rn(t, t));
        }
        r2 = fmax(r2, s);
    }
    for (int o = 16; o > 0; o >>= 1) r2 = fmax(r2, __shfl_xor_sync(0xFFFFFFFFu, r2, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&out->r2, (unsigned long long)__double_as_longlong(r2));
}

cudaError_t launch_mesh_bounds(const float4* pos, uint32_t n, MeshBounds* out, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(out->lo, 0xFF, sizeof(out->lo), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(out->hi, 0, sizeof(out->hi) + sizeof(out->r2), stream);
    if (e != cudaSuccess || n == 0) return e;
    const unsigned g = grid_for(n, 256, 1024);
    mesh_box_kernel<<<g, 256, 0, stream>>>(pos, n, out);
    mesh_radius_kernel<<<g, 256, 0, stream>>>(pos, n, out);
    return cudaGetLastError();
}

float mesh_bounds_float(uint32_t o) {
    const uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    float f;
    std::memcpy(&f, &u, sizeof(f));
    return f;
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
