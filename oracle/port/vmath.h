/* Oracle test infrastructure: float vector math for the C restatement of the AxiomR
 * draw path. Each function rounds in the order the oracle's glm-compatible header
 * (oracle/shim/glm/glm.hpp) documents, so this port and the reference compiled against
 * that header agree bit for bit:
 *   dot3 = (ax*bx + ay*by) + az*bz;  dot4 = (ax*bx + ay*by) + (az*bz + aw*bw)
 *   mat3*v = (c0*x + c1*y) + c2*z;   mat4*v = (c0*x + c1*y) + (c2*z + c3*w)
 *   normalize(v) = v * (1 / sqrt(dot(v, v)));  mix(x, y, a) = x*(1-a) + y*a
 * Build with -ffp-contract=off (oracle/build.py) so no multiply-add is fused. */
#ifndef AXO_VMATH_H
#define AXO_VMATH_H
#include <math.h>

typedef struct { float x, y; } v2;
typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;
typedef struct { v4 c[4]; } m4; /* column-major: c[col].{x,y,z,w} = rows 0..3 */
typedef struct { v3 c[3]; } m3;

static inline v2 V2(float x, float y) { v2 r = {x, y}; return r; }
static inline v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v4 V4(float x, float y, float z, float w) { v4 r = {x, y, z, w}; return r; }

static inline v2 add2(v2 a, v2 b) { return V2(a.x + b.x, a.y + b.y); }
static inline v2 mul2s(v2 a, float s) { return V2(a.x * s, a.y * s); }
static inline v2 smul2(float s, v2 a) { return V2(s * a.x, s * a.y); }
static inline v2 div2s(v2 a, float s) { return V2(a.x / s, a.y / s); }

static inline v3 add3(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 div3(v3 a, v3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 mul3s(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline v3 smul3(float s, v3 a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline v3 div3s(v3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline v3 add3s(v3 a, float s) { return V3(a.x + s, a.y + s, a.z + s); }
static inline v3 sub3s(v3 a, float s) { return V3(a.x - s, a.y - s, a.z - s); }
static inline v3 neg3(v3 a) { return V3(-a.x, -a.y, -a.z); }
static inline float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 normalize3(v3 v) { return mul3s(v, 1.0f / sqrtf(dot3(v, v))); }
static inline v3 cross3(v3 a, v3 b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 mix3(v3 x, v3 y, float a) { return add3(mul3s(x, 1.0f - a), mul3s(y, a)); }
static inline v2 mix2(v2 x, v2 y, float a) { return add2(mul2s(x, 1.0f - a), mul2s(y, a)); }
static inline float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
/* reflect(I, N) = I - (2*dot(N, I)) * N */
static inline v3 reflect3(v3 i, v3 n) { return sub3(i, smul3(2.0f * dot3(n, i), n)); }
static inline v3 pow3(v3 b, v3 e) { return V3(powf(b.x, e.x), powf(b.y, e.y), powf(b.z, e.z)); }
/* std::max(a, b) / std::min(a, b) / std::clamp(v, lo, hi) semantics (NaN follows them) */
static inline float maxf_std(float a, float b) { return (a < b) ? b : a; }
static inline float minf_std(float a, float b) { return (b < a) ? b : a; }
static inline float clampf_std(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

static inline v4 add4(v4 a, v4 b) { return V4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline v4 mul4s(v4 a, float s) { return V4(a.x * s, a.y * s, a.z * s, a.w * s); }
static inline v4 mix4(v4 x, v4 y, float a) { return add4(mul4s(x, 1.0f - a), mul4s(y, a)); }
static inline v3 xyz(v4 a) { return V3(a.x, a.y, a.z); }

static inline v4 m4v(const m4* m, v4 v) {
    return add4(add4(mul4s(m->c[0], v.x), mul4s(m->c[1], v.y)), add4(mul4s(m->c[2], v.z), mul4s(m->c[3], v.w)));
}
static inline m4 m4m(const m4* a, const m4* b) {
    m4 r;
    for (int j = 0; j < 4; ++j) r.c[j] = m4v(a, b->c[j]);
    return r;
}
static inline v3 m3v(const m3* m, v3 v) {
    return add3(add3(mul3s(m->c[0], v.x), mul3s(m->c[1], v.y)), mul3s(m->c[2], v.z));
}
static inline m4 m4_load(const float* f) {
    m4 r;
    for (int j = 0; j < 4; ++j) r.c[j] = V4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
    return r;
}
static inline void m4_store(const m4* m, float* f) {
    for (int j = 0; j < 4; ++j) {
        f[4 * j] = m->c[j].x; f[4 * j + 1] = m->c[j].y; f[4 * j + 2] = m->c[j].z; f[4 * j + 3] = m->c[j].w;
    }
}
static inline float m4_at(const m4* m, int row, int col) {
    const v4* c = &m->c[col];
    return row == 0 ? c->x : (row == 1 ? c->y : (row == 2 ? c->z : c->w));
}

/* mat4 inverse by the adjugate with complementary 2x2 minors, in the order the oracle
 * header documents (oracle/shim/glm/glm.hpp, inverse). */
m4 m4_inverse(const m4* m);

#endif
