/* Oracle test infrastructure: homogeneous clipping, triangle setup and backface test,
 * restating reference src/pipeline.cpp:176-228 (clipTriangle), 243-272
 * (interpolateVertices), 274-285 (distFunc), 302-370 (clipTriangleSinglePlane) and
 * src/tiled_pipeline.cpp:15-23 (clampW), 53-72 (Triangle ctor), 89-119 (isBackface). */
#include <string.h>

#include "axo_port.h"

/* pipeline.cpp:274-285 */
static float dist_plane(v4 v, int plane) {
    switch (plane) {
        case 0: return v.x + v.w;
        case 1: return v.w - v.x;
        case 2: return v.y + v.w;
        case 3: return v.w - v.y;
        case 4: return v.z + v.w;
        case 5: return v.w - v.z;
        default: return 0.0f;
    }
}

/* pipeline.cpp:243-272: attributes by glm::mix, directions re-normalised, uv mixed with
 * w weights and divided by the mixed w. */
static cvert interpolate(const cvert* a, const cvert* b, float t) {
    cvert o;
    o.pos = mix3(a->pos, b->pos, t);
    o.nrm = normalize3(mix3(a->nrm, b->nrm, t));
    o.tan = normalize3(mix3(a->tan, b->tan, t));
    o.bit = normalize3(mix3(a->bit, b->bit, t));
    o.clip = mix4(a->clip, b->clip, t);
    float w0 = a->clip.w, w1 = b->clip.w;
    v2 uv0w = mul2s(a->uv, w0);
    v2 uv1w = mul2s(b->uv, w1);
    v2 iuv = mix2(uv0w, uv1w, t);
    float iw = mixf(w0, w1, t);
    o.uv = div2s(iuv, iw);
    return o;
}

static float clip_t(float dn, float dd) {
    float denom = dn - dd;
    return (fabsf(denom) < 1e-7f) ? 0.5f : (dn / denom);
}

/* pipeline.cpp:302-370 (McGuire-style single-plane clip); returns 0, 3 or 4 */
static int clip_single_plane(int plane, cvert* v0, cvert* v1, cvert* v2, cvert* v3) {
    float d0 = dist_plane(v0->clip, plane);
    float d1 = dist_plane(v1->clip, plane);
    float d2 = dist_plane(v2->clip, plane);
    if (d0 < 0.f && d1 < 0.f && d2 < 0.f) return 0;
    if (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f) {
        *v3 = *v0;
        return 3;
    }
    cvert tv;
    float td;
    if ((d1 >= 0.f) && !(d0 >= 0.f)) {
        /* rotate (v0, v1, v2) <- (v1, v2, v0) */
        tv = *v0; *v0 = *v1; *v1 = tv; td = d0; d0 = d1; d1 = td;
        tv = *v1; *v1 = *v2; *v2 = tv; td = d1; d1 = d2; d2 = td;
    } else if ((d2 >= 0.f) && !(d1 >= 0.f)) {
        /* rotate (v0, v1, v2) <- (v2, v0, v1) */
        tv = *v2; *v2 = *v1; *v1 = tv; td = d2; d2 = d1; d1 = td;
        tv = *v1; *v1 = *v0; *v0 = tv; td = d1; d1 = d0; d0 = td;
    }
    float t02 = clip_t(d0, d2);
    *v3 = interpolate(v0, v2, t02);
    if (d1 >= 0.f) {
        float t12 = clip_t(d1, d2);
        *v2 = interpolate(v1, v2, t12);
        return 4;
    }
    float t01 = clip_t(d0, d1);
    *v1 = interpolate(v0, v1, t01);
    *v2 = *v3;
    return 3;
}

/* pipeline.cpp:176-228: six planes in order; a result that would overflow the 24-vertex
 * array is dropped whole. Returns the output vertex count (a multiple of 3). */
int port_clip(cvert* out, int count) {
    cvert next[MAX_CLIPPED_VERTS];
    int index = count;
    for (int plane = 0; plane < 6; ++plane) {
        int n = 0;
        for (int i = 0; i < index; i += 3) {
            cvert v0 = out[i], v1 = out[i + 1], v2 = out[i + 2], v3;
            int r = clip_single_plane(plane, &v0, &v1, &v2, &v3);
            if (r == 3) {
                if (n + 3 <= MAX_CLIPPED_VERTS) {
                    next[n] = v0; next[n + 1] = v1; next[n + 2] = v2;
                    n += 3;
                }
            } else if (r == 4) {
                if (n + 6 <= MAX_CLIPPED_VERTS) {
                    next[n] = v0; next[n + 1] = v1; next[n + 2] = v2;
                    next[n + 3] = v0; next[n + 4] = v2; next[n + 5] = v3;
                    n += 6;
                }
            }
        }
        index = n;
        memcpy(out, next, sizeof(cvert) * (size_t)n);
        if (index == 0) break;
    }
    return index;
}

/* tiled_pipeline.cpp:15-23 */
static float clamp_w(float w) {
    const float tiny = 1e-6f;
    if (fabsf(w) < tiny) w = (w < 0.0f) ? -tiny : tiny;
    return w;
}

static v2 screen_pos(v4 c, int width, int height, float* ndcz) {
    float w = clamp_w(c.w);
    float inv = 1.0f / w;
    if (ndcz) *ndcz = c.z * inv;
    return V2(((c.x * inv) + 1.0f) * 0.5f * (float)width, ((c.y * inv) + 1.0f) * 0.5f * (float)height);
}

/* tiled_pipeline.cpp:53-72: screenPos[6], ndcZ[3], minX, minY, maxX, maxY with
 * std::min/max over initializer lists (first of equals wins, NaN follows '<'). */
void port_setup(const cvert* v, int width, int height, float* o) {
    v2 s[3];
    float z[3];
    for (int i = 0; i < 3; ++i) s[i] = screen_pos(v[i].clip, width, height, &z[i]);
    float mnx = s[0].x, mny = s[0].y, mxx = s[0].x, mxy = s[0].y;
    for (int i = 1; i < 3; ++i) {
        if (s[i].x < mnx) mnx = s[i].x;
        if (s[i].y < mny) mny = s[i].y;
        if (mxx < s[i].x) mxx = s[i].x;
        if (mxy < s[i].y) mxy = s[i].y;
    }
    o[0] = s[0].x; o[1] = s[0].y; o[2] = s[1].x; o[3] = s[1].y; o[4] = s[2].x; o[5] = s[2].y;
    o[6] = z[0]; o[7] = z[1]; o[8] = z[2];
    o[9] = mnx; o[10] = mny; o[11] = mxx; o[12] = mxy;
}

/* tiled_pipeline.cpp:89-119: culled when the screen-space signed area is negative */
int port_backface(const cvert* a, const cvert* b, const cvert* c, int width, int height) {
    v2 p0 = screen_pos(a->clip, width, height, 0);
    v2 p1 = screen_pos(b->clip, width, height, 0);
    v2 p2 = screen_pos(c->clip, width, height, 0);
    float dx1 = p1.x - p0.x, dy1 = p1.y - p0.y;
    float dx2 = p2.x - p0.x, dy2 = p2.y - p0.y;
    float area = dx1 * dy2 - dx2 * dy1;
    return area < 0;
}

static cvert load_cv(const float* f) {
    cvert c;
    c.pos = V3(f[0], f[1], f[2]);
    c.uv = V2(f[3], f[4]);
    c.nrm = V3(f[5], f[6], f[7]);
    c.tan = V3(f[8], f[9], f[10]);
    c.bit = V3(f[11], f[12], f[13]);
    c.clip = V4(f[14], f[15], f[16], f[17]);
    return c;
}

static void store_cv(const cvert* c, float* f) {
    float v[18] = {c->pos.x, c->pos.y, c->pos.z, c->uv.x, c->uv.y, c->nrm.x, c->nrm.y, c->nrm.z,
                   c->tan.x, c->tan.y, c->tan.z, c->bit.x, c->bit.y, c->bit.z,
                   c->clip.x, c->clip.y, c->clip.z, c->clip.w};
    memcpy(f, v, sizeof(v));
}

int port_clip_triangle(const float* in3, float* out24, int* count) {
    cvert v[MAX_CLIPPED_VERTS];
    for (int k = 0; k < 3; ++k) v[k] = load_cv(in3 + AXO_CV_FLOATS * k);
    int n = port_clip(v, 3);
    for (int k = 0; k < n; ++k) store_cv(&v[k], out24 + AXO_CV_FLOATS * k);
    *count = n;
    return 0;
}

int port_triangle(const float* in3, int width, int height, float* out13, int* backface) {
    cvert v[3];
    for (int k = 0; k < 3; ++k) v[k] = load_cv(in3 + AXO_CV_FLOATS * k);
    *backface = port_backface(&v[0], &v[1], &v[2], width, height);
    port_setup(v, width, height, out13);
    return 0;
}
