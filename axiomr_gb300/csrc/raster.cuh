// Clipping, triangle setup and per-pixel coverage/depth for the draw kernels.
//
// Every function reproduces the reference's arithmetic exactly (see fmath.cuh):
//   clip_triangle      src/pipeline.cpp:176-228, 243-272, 274-285, 302-370
//   screen_setup       src/tiled_pipeline.cpp:15-23 (clampW), 53-72 (Triangle ctor),
//                      89-119 (isBackface)
//   edge_setup         src/tiled_pipeline.cpp:436-487 (edge terms, area test, sign flip)
//   eval_pixel         src/tiled_pipeline.cpp:502-562 (row start, 8-pixel steps, lane
//                      offsets, barycentrics, depth)
// The reference evaluates a triangle's edge functions from the first column of each
// 16-pixel tile it covers, stepping in 8-pixel blocks; eval_pixel derives that start
// column from the pixel itself, so any thread can evaluate any pixel independently and
// still obtain the reference's bits.
#pragma once
#include "device_types.h"
#include "fmath.cuh"

namespace axr {

// ------------------------------------------------------------------ clipped vertices
enum : int { kAttrPos = 1, kAttrUv = 2, kAttrNrm = 4, kAttrTanBit = 8 };

struct CVClip {
    f4 clip;
};
struct CVFull {
    f4 clip;
    f3 pos;
    f2 uv;
    f3 nrm, tan, bit;
};

template <int A, class CV>
__device__ __forceinline__ CV interpolate(const CV& a, const CV& b, float t) {
    CV o;
    o.clip = mix(a.clip, b.clip, t);
    if constexpr (A != 0) {
        if constexpr ((A & kAttrPos) != 0) o.pos = mix(a.pos, b.pos, t);
        if constexpr ((A & kAttrNrm) != 0) o.nrm = normalize(mix(a.nrm, b.nrm, t));
        if constexpr ((A & kAttrTanBit) != 0) {
            o.tan = normalize(mix(a.tan, b.tan, t));
            o.bit = normalize(mix(a.bit, b.bit, t));
        }
        if constexpr ((A & kAttrUv) != 0) {
            float w0 = a.clip.w, w1 = b.clip.w;
            f2 iuv = mix(mul(a.uv, w0), mul(b.uv, w1), t);
            o.uv = divs(iuv, mix(w0, w1, t));
        }
    }
    return o;
}

__device__ __forceinline__ float plane_dist(f4 v, int plane) {
    switch (plane) {
        case 0: return fadd(v.x, v.w);
        case 1: return fsub(v.w, v.x);
        case 2: return fadd(v.y, v.w);
        case 3: return fsub(v.w, v.y);
        case 4: return fadd(v.z, v.w);
        default: return fsub(v.w, v.z);
    }
}

__device__ __forceinline__ float clip_t(float dn, float dd) {
    float denom = fsub(dn, dd);
    return (fabsf(denom) < 1e-7f) ? 0.5f : fdiv(dn, denom);
}

template <class T>
__device__ __forceinline__ void swap_(T& a, T& b) {
    T t = a;
    a = b;
    b = t;
}

// One plane; returns 0 (all outside), 3 (triangle v0 v1 v2) or 4 (quad v0 v1 v2 v3).
template <int A, class CV>
__device__ int clip_plane(int plane, CV& v0, CV& v1, CV& v2, CV& v3) {
    float d0 = plane_dist(v0.clip, plane), d1 = plane_dist(v1.clip, plane), d2 = plane_dist(v2.clip, plane);
    if (d0 < 0.f && d1 < 0.f && d2 < 0.f) return 0;
    if (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f) {
        v3 = v0;
        return 3;
    }
    if ((d1 >= 0.f) && !(d0 >= 0.f)) {
        swap_(v0, v1); swap_(d0, d1);
        swap_(v1, v2); swap_(d1, d2);
    } else if ((d2 >= 0.f) && !(d1 >= 0.f)) {
        swap_(v2, v1); swap_(d2, d1);
        swap_(v1, v0); swap_(d1, d0);
    }
    v3 = interpolate<A>(v0, v2, clip_t(d0, d2));
    if (d1 >= 0.f) {
        v2 = interpolate<A>(v1, v2, clip_t(d1, d2));
        return 4;
    }
    v1 = interpolate<A>(v0, v1, clip_t(d0, d1));
    v2 = v3;
    return 3;
}

// Six planes in order over a 24-vertex ping-pong pair; a result that would overflow 24
// vertices is dropped whole, as in the reference. Input in buf_a[0..2]; returns the
// vertex count and sets *out to the buffer holding the result.
template <int A, class CV>
__device__ int clip_triangle(CV* buf_a, CV* buf_b, CV** out) {
    CV* cur = buf_a;
    CV* nxt = buf_b;
    int n = 3;
    for (int plane = 0; plane < 6; ++plane) {
        int m = 0;
        for (int i = 0; i < n; i += 3) {
            CV v0 = cur[i], v1 = cur[i + 1], v2 = cur[i + 2], v3;
            int r = clip_plane<A>(plane, v0, v1, v2, v3);
            if (r == 3) {
                if (m + 3 <= kMaxClipVerts) {
                    nxt[m] = v0; nxt[m + 1] = v1; nxt[m + 2] = v2;
                    m += 3;
                }
            } else if (r == 4) {
                if (m + 6 <= kMaxClipVerts) {
                    nxt[m] = v0; nxt[m + 1] = v1; nxt[m + 2] = v2;
                    nxt[m + 3] = v0; nxt[m + 4] = v2; nxt[m + 5] = v3;
                    m += 6;
                }
            }
        }
        CV* t = cur;
        cur = nxt;
        nxt = t;
        n = m;
        if (n == 0) break;
    }
    *out = cur;
    return n;
}

// Trivial cases of clip_triangle without running it: returns 3 when every plane keeps
// all three vertices (output = input), 0 when the first plane that does not keep all
// three rejects all three (output empty), and -1 when the general clipper must run.
__device__ __forceinline__ int clip_classify(f4 c0, f4 c1, f4 c2) {
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        float d0 = plane_dist(c0, p), d1 = plane_dist(c1, p), d2 = plane_dist(c2, p);
        if (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f) continue;
        if (d0 < 0.f && d1 < 0.f && d2 < 0.f) return 0;
        return -1;
    }
    return 3;
}

// ------------------------------------------------------------------ setup
struct Screen {
    float x[3], y[3], z[3];
    float minx, miny, maxx, maxy;
};

__device__ __forceinline__ float clamp_w(float w) {
    const float tiny = 1e-6f;
    if (fabsf(w) < tiny) w = (w < 0.0f) ? -tiny : tiny;
    return w;
}

// Screen position and NDC depth of one clip-space vertex (Triangle ctor, per vertex).
__device__ __forceinline__ f3 screen_vertex(f4 c, float fw, float fh) {
    float inv = frcp(clamp_w(c.w));
    return mk3(fmul(fmul(fadd(fmul(c.x, inv), 1.0f), 0.5f), fw), fmul(fmul(fadd(fmul(c.y, inv), 1.0f), 0.5f), fh),
               fmul(c.z, inv));
}

// Bounding box with std::min / std::max over an initializer list: the first of equal
// values wins and NaN follows operator<.
__device__ __forceinline__ void screen_bbox(Screen& s) {
    s.minx = s.x[0]; s.miny = s.y[0]; s.maxx = s.x[0]; s.maxy = s.y[0];
#pragma unroll
    for (int k = 1; k < 3; ++k) {
        if (s.x[k] < s.minx) s.minx = s.x[k];
        if (s.y[k] < s.miny) s.miny = s.y[k];
        if (s.maxx < s.x[k]) s.maxx = s.x[k];
        if (s.maxy < s.y[k]) s.maxy = s.y[k];
    }
}

__device__ __forceinline__ void screen_setup(f4 c0, f4 c1, f4 c2, int width, int height, Screen& s) {
    const f4 c[3] = {c0, c1, c2};
    const float fw = (float)width, fh = (float)height;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f3 v = screen_vertex(c[k], fw, fh);
        s.x[k] = v.x;
        s.y[k] = v.y;
        s.z[k] = v.z;
    }
    screen_bbox(s);
}

// Per-vertex clip-plane classification: bit p set when the vertex is inside plane p
// (distance >= 0), bit 6+p set when it is outside (distance < 0); a NaN distance sets
// neither, as the reference's comparisons treat it.
__device__ __forceinline__ uint32_t plane_masks(f4 c) {
    uint32_t m = 0;
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        float d = plane_dist(c, p);
        if (d >= 0.f) m |= 1u << p;
        if (d < 0.f) m |= 1u << (6 + p);
    }
    return m;
}

// clip_classify from per-vertex masks.
__device__ __forceinline__ int classify_masks(uint32_t m0, uint32_t m1, uint32_t m2) {
    const uint32_t all = m0 & m1 & m2;
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        if (all & (1u << p)) continue;
        if (all & (1u << (6 + p))) return 0;
        return -1;
    }
    return 3;
}

__device__ __forceinline__ bool is_backface(const Screen& s) {
    float dx1 = fsub(s.x[1], s.x[0]), dy1 = fsub(s.y[1], s.y[0]);
    float dx2 = fsub(s.x[2], s.x[0]), dy2 = fsub(s.y[2], s.y[0]);
    return fsub(fmul(dx1, dy2), fmul(dx2, dy1)) < 0.0f;
}

// Edge functions after the reference's sign normalisation; valid=false when the
// reference's raster returns before touching a pixel (empty box or 0 <= area < 1e-12).
struct Edges {
    float a[3], b[3], c[3];
    float inv_area;
    float z[3];
    int x_lo, x_hi, y_lo, y_hi;  // covered pixel range [lo, hi) clipped to the target
};

// `(double)area < 1e-12` for a float area holds exactly when area <= 1e-12f
// (1e-12f = 0x1.197998p-40 lies just below 1e-12 and its successor just above).
constexpr float kAreaEpsilon = 1e-12f;

__device__ __forceinline__ bool edge_setup(const Screen& s, int width, int height, Edges& e) {
    int bx0 = __float2int_rz(floorf(s.minx)), by0 = __float2int_rz(floorf(s.miny));
    int bx1 = __float2int_rz(ceilf(s.maxx)), by1 = __float2int_rz(ceilf(s.maxy));
    e.x_lo = max(0, bx0);
    e.y_lo = max(0, by0);
    e.x_hi = min(width, bx1);
    e.y_hi = min(height, by1);
    if (e.x_lo >= e.x_hi || e.y_lo >= e.y_hi) return false;
    const float x0 = s.x[0], y0 = s.y[0], x1 = s.x[1], y1 = s.y[1], x2 = s.x[2], y2 = s.y[2];
    float c0 = fsub(fmul(x1, y2), fmul(x2, y1));
    float c1 = fsub(fmul(x2, y0), fmul(x0, y2));
    float c2 = fsub(fmul(x0, y1), fmul(x1, y0));
    float area = fadd(fadd(c0, c1), c2);
    if (area >= 0.0f && area <= kAreaEpsilon) return false;
    float a0 = fsub(y1, y2), b0 = fsub(x2, x1);
    float a1 = fsub(y2, y0), b1 = fsub(x0, x2);
    float a2 = fsub(y0, y1), b2 = fsub(x1, x0);
    if (area < 0.0f) {
        a0 = -a0; b0 = -b0; c0 = -c0;
        a1 = -a1; b1 = -b1; c1 = -c1;
        a2 = -a2; b2 = -b2; c2 = -c2;
        area = -area;
    }
    e.a[0] = a0; e.b[0] = b0; e.c[0] = c0;
    e.a[1] = a1; e.b[1] = b1; e.c[1] = c1;
    e.a[2] = a2; e.b[2] = b2; e.c[2] = c2;
    e.inv_area = frcp(area);
    e.z[0] = s.z[0]; e.z[1] = s.z[1]; e.z[2] = s.z[2];
    return true;
}

// Coverage and depth of pixel (px, py), px in [x_lo, x_hi), py in [y_lo, y_hi).
// The reference starts each row at column sx = max(tile start, floor(minX)) of the
// pixel's 16-pixel tile, adds a*8 once per 8-pixel block and a*lane inside the block.
struct PixelEval {
    bool covered;
    float z, alpha, beta, gamma;
};

__device__ __forceinline__ PixelEval eval_pixel(const Edges& e, int px, int py) {
    int sx = max(px & ~(kTile - 1), e.x_lo);
    int i = px - sx;
    float fsx = fadd((float)sx, 0.5f);
    float fpy = fadd((float)py, 0.5f);
    float lane = (float)(i & 7);
    float cov[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float row = fadd(fadd(fmul(e.a[k], fsx), fmul(e.b[k], fpy)), e.c[k]);
        if (i >= 8) row = fadd(row, fmul(e.a[k], 8.0f));
        cov[k] = fadd(row, fmul(e.a[k], lane));
    }
    PixelEval r;
    r.covered = cov[0] >= 0.f && cov[1] >= 0.f && cov[2] >= 0.f;
    r.alpha = fmul(cov[0], e.inv_area);
    r.beta = fmul(cov[1], e.inv_area);
    r.gamma = fmul(cov[2], e.inv_area);
    r.z = fadd(fadd(fmul(e.z[0], r.alpha), fmul(e.z[1], r.beta)), fmul(e.z[2], r.gamma));
    return r;
}

// ------------------------------------------------------------------ mesh access
struct FaceRef {
    uint32_t face;
    uint32_t material;
};

// Draw-order position -> (face, material) through the material groups.
__device__ __forceinline__ FaceRef face_of(const DevMesh& m, uint32_t ordinal) {
    uint32_t k = 0;
    while (k + 1 < m.num_groups && ordinal >= m.groups[k].base + m.groups[k].count) ++k;
    const DevGroup g = m.groups[k];
    return {g.start + (ordinal - g.base), g.material};
}

__device__ __forceinline__ f4 load_clip(const DevMesh& m, const float* mvp, uint32_t vi) {
    float4 p = __ldg(&m.pos[vi]);
    return mat4_mul(mvp, p.x, p.y, p.z, 1.0f);
}

__device__ __forceinline__ uint3 load_face(const DevMesh& m, uint32_t face) {
    const uint32_t* p = m.idx + 3ull * face;
    return make_uint3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

}  // namespace axr
