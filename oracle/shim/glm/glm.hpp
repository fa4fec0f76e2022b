// Oracle test infrastructure: a glm-compatible vector/matrix/quaternion header written
// for this project. It exists only so that the AxiomR reference sources (which include
// glm, a dependency that is not vendored in the reference tree and has no pinned
// version) can be compiled unmodified as the CPU oracle. It is written from the
// documented GLSL / glm semantics (column-major matrices, GLSL built-in functions,
// Hamilton quaternions, the OpenGL perspective matrix) and does not reproduce glm's own
// source.
//
// Every floating-point result depends on the association order of sums, so each
// operation below states its order. The CUDA path and the C restatement in
// oracle/port follow exactly these orders:
//   * component-wise ops: one IEEE op per component;
//   * dot(vec3): (a.x*b.x + a.y*b.y) + a.z*b.z          (left to right)
//   * dot(vec4), dot(quat): (x*x' + y*y') + (z*z' + w*w') (pairwise)
//   * mat3 * vec3: (c0*v.x + c1*v.y) + c2*v.z            (left to right)
//   * mat4 * vec4: (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w) (pairwise)
//   * mat4 * mat4: column j of the result = A * B[j] (as above)
//   * normalize(v) = v * (1 / sqrt(dot(v, v)))
//   * mix(x, y, a) = x * (1 - a) + y * a                  (GLSL definition)
//   * reflect(I, N) = I - (2 * dot(N, I)) * N             (GLSL definition)
//   * cross(a, b) = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   * clamp(x, lo, hi) = min(max(x, lo), hi)              (GLSL definition)
// Parity against upstream glm is not pinned: the reference ships no tests and no glm
// copy, so "bit-exact" means bit-exact against the reference compiled with this header.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstddef>
#include <algorithm>
#include <memory>
#include <string>
#include <iostream>
#if defined(__x86_64__) || defined(__i386__)
#include <immintrin.h>  // the reference's raster loops use AVX intrinsics without including this
#endif

namespace glm {

template <typename T> constexpr T pi() { return static_cast<T>(3.14159265358979323846264338327950288); }

constexpr float radians(float degrees) { return degrees * 0.0174532925199432957692369076848861f; }
constexpr float degrees(float radians) { return radians * 57.2957795130823208767981548141052f; }
inline float abs(float x) { return std::fabs(x); }
inline float asin(float x) { return std::asin(x); }
inline float acos(float x) { return std::acos(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float min(float a, float b) { return (b < a) ? b : a; }
inline float max(float a, float b) { return (a < b) ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }

// ---------------------------------------------------------------- vectors
struct vec2 {
    union { float x; float r; float s; };
    union { float y; float g; float t; };
    constexpr vec2() : x(0.0f), y(0.0f) {}
    constexpr explicit vec2(float v) : x(v), y(v) {}
    constexpr vec2(float a, float b) : x(a), y(b) {}
    static constexpr int length() { return 2; }
    float& operator[](int i) { return i == 0 ? x : y; }
    const float& operator[](int i) const { return i == 0 ? x : y; }
    vec2& operator+=(const vec2& o) { x += o.x; y += o.y; return *this; }
    vec2& operator-=(const vec2& o) { x -= o.x; y -= o.y; return *this; }
    vec2& operator*=(float s) { x *= s; y *= s; return *this; }
};
inline vec2 operator+(const vec2& a, const vec2& b) { return {a.x + b.x, a.y + b.y}; }
inline vec2 operator-(const vec2& a, const vec2& b) { return {a.x - b.x, a.y - b.y}; }
inline vec2 operator*(const vec2& a, const vec2& b) { return {a.x * b.x, a.y * b.y}; }
inline vec2 operator/(const vec2& a, const vec2& b) { return {a.x / b.x, a.y / b.y}; }
inline vec2 operator*(const vec2& a, float s) { return {a.x * s, a.y * s}; }
inline vec2 operator*(float s, const vec2& a) { return {s * a.x, s * a.y}; }
inline vec2 operator/(const vec2& a, float s) { return {a.x / s, a.y / s}; }
inline vec2 operator-(const vec2& a) { return {-a.x, -a.y}; }
inline bool operator==(const vec2& a, const vec2& b) { return a.x == b.x && a.y == b.y; }
inline bool operator!=(const vec2& a, const vec2& b) { return !(a == b); }

struct vec4;
struct vec3 {
    union { float x; float r; float s; };
    union { float y; float g; float t; };
    union { float z; float b; float p; };
    constexpr vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    constexpr explicit vec3(float v) : x(v), y(v), z(v) {}
    constexpr vec3(float a, float b_, float c) : x(a), y(b_), z(c) {}
    explicit vec3(const vec4& v);
    static constexpr int length() { return 3; }  // glm semantics: number of components
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};
inline vec3 operator+(const vec3& a, const vec3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(const vec3& a, const vec3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(const vec3& a, const vec3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator/(const vec3& a, const vec3& b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline vec3 operator+(const vec3& a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline vec3 operator-(const vec3& a, float s) { return {a.x - s, a.y - s, a.z - s}; }
inline vec3 operator*(const vec3& a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator*(float s, const vec3& a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec3 operator/(const vec3& a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline vec3 operator-(const vec3& a) { return {-a.x, -a.y, -a.z}; }
inline bool operator==(const vec3& a, const vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const vec3& a, const vec3& b) { return !(a == b); }

struct vec4 {
    union { float x; float r; float s; };
    union { float y; float g; float t; };
    union { float z; float b; float p; };
    union { float w; float a; float q; };
    constexpr vec4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
    constexpr explicit vec4(float v) : x(v), y(v), z(v), w(v) {}
    constexpr vec4(float a_, float b_, float c, float d) : x(a_), y(b_), z(c), w(d) {}
    constexpr vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    static constexpr int length() { return 4; }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    vec4& operator+=(const vec4& o) { x += o.x; y += o.y; z += o.z; w += o.w; return *this; }
    vec4& operator*=(float s) { x *= s; y *= s; z *= s; w *= s; return *this; }
};
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}
inline vec4 operator+(const vec4& a, const vec4& b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline vec4 operator-(const vec4& a, const vec4& b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline vec4 operator*(const vec4& a, const vec4& b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
inline vec4 operator*(const vec4& a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
inline vec4 operator*(float s, const vec4& a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }
inline vec4 operator/(const vec4& a, float s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }
inline vec4 operator-(const vec4& a) { return {-a.x, -a.y, -a.z, -a.w}; }
inline bool operator==(const vec4& a, const vec4& b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

struct ivec2 {
    int x, y;
    constexpr ivec2() : x(0), y(0) {}
    constexpr explicit ivec2(int v) : x(v), y(v) {}
    constexpr ivec2(int a, int b) : x(a), y(b) {}
};
struct uvec2 {
    unsigned x, y;
    constexpr uvec2() : x(0), y(0) {}
    constexpr uvec2(unsigned a, unsigned b) : x(a), y(b) {}
};

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
inline float length2(const vec3& v) { return dot(v, v); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec2 normalize(const vec2& v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline vec3 normalize(const vec3& v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline vec4 normalize(const vec4& v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline vec2 mix(const vec2& x, const vec2& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec4 mix(const vec4& x, const vec4& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 reflect(const vec3& i, const vec3& n) { return i - (2.0f * dot(n, i)) * n; }
inline vec3 pow(const vec3& b, const vec3& e) { return {std::pow(b.x, e.x), std::pow(b.y, e.y), std::pow(b.z, e.z)}; }
inline vec3 min(const vec3& a, const vec3& b) { return {min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)}; }
inline vec3 max(const vec3& a, const vec3& b) { return {max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)}; }
inline vec3 clamp(const vec3& x, float lo, float hi) { return {clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi)}; }
inline vec3 abs(const vec3& v) { return {std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)}; }
inline float compMax(const vec3& v) { return max(max(v.x, v.y), v.z); }
inline float compMin(const vec3& v) { return min(min(v.x, v.y), v.z); }

// ---------------------------------------------------------------- matrices (column-major)
struct mat4;
struct mat3 {
    vec3 c[3];
    constexpr mat3() : c{vec3(1, 0, 0), vec3(0, 1, 0), vec3(0, 0, 1)} {}
    constexpr explicit mat3(float d) : c{vec3(d, 0, 0), vec3(0, d, 0), vec3(0, 0, d)} {}
    constexpr mat3(const vec3& a, const vec3& b, const vec3& d) : c{a, b, d} {}
    explicit mat3(const mat4& m);
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3& m, const vec3& v) { return (m[0] * v.x + m[1] * v.y) + m[2] * v.z; }
inline mat3 operator*(float s, const mat3& m) { return {s * m[0], s * m[1], s * m[2]}; }
inline mat3 operator*(const mat3& m, float s) { return {m[0] * s, m[1] * s, m[2] * s}; }
inline mat3 operator+(const mat3& a, const mat3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline mat3 operator*(const mat3& a, const mat3& b) { return {a * b[0], a * b[1], a * b[2]}; }

struct mat4 {
    vec4 c[4];
    constexpr mat4() : c{vec4(1, 0, 0, 0), vec4(0, 1, 0, 0), vec4(0, 0, 1, 0), vec4(0, 0, 0, 1)} {}
    constexpr explicit mat4(float d) : c{vec4(d, 0, 0, 0), vec4(0, d, 0, 0), vec4(0, 0, d, 0), vec4(0, 0, 0, d)} {}
    constexpr mat4(const vec4& a, const vec4& b, const vec4& d, const vec4& e) : c{a, b, d, e} {}
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline mat3::mat3(const mat4& m) : c{vec3(m[0]), vec3(m[1]), vec3(m[2])} {}
inline vec4 operator*(const mat4& m, const vec4& v) {
    return (m[0] * v.x + m[1] * v.y) + (m[2] * v.z + m[3] * v.w);
}
inline mat4 operator*(const mat4& a, const mat4& b) { return {a * b[0], a * b[1], a * b[2], a * b[3]}; }

inline mat4 transpose(const mat4& m) {
    mat4 r(0.0f);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r[i][j] = m[j][i];
    return r;
}
inline mat3 transpose(const mat3& m) {
    mat3 r(0.0f);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i][j] = m[j][i];
    return r;
}

// Inverse by the adjugate (Laplace expansion over complementary 2x2 minors). With
// a[i][j] = row i, column j, the 2x2 minors of rows 0-1 (s*) and rows 2-3 (t*) are
//   s0 = a00*a11 - a10*a01, s1 = a00*a12 - a10*a02, s2 = a00*a13 - a10*a03,
//   s3 = a01*a12 - a11*a02, s4 = a01*a13 - a11*a03, s5 = a02*a13 - a12*a03,
//   t0 = a20*a31 - a30*a21, t1 = a20*a32 - a30*a22, t2 = a20*a33 - a30*a23,
//   t3 = a21*a32 - a31*a22, t4 = a21*a33 - a31*a23, t5 = a22*a33 - a32*a23,
//   det = ((s0*t5 - s1*t4) + (s2*t3 + s3*t2)) - (s4*t1 - s5*t0),
// and each adjugate entry is a signed three-term sum evaluated left to right, scaled
// by invDet = 1 / det.
inline mat4 inverse(const mat4& m) {
    auto a = [&](int row, int col) { return m[col][row]; };
    float s0 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1);
    float s1 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
    float s2 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3);
    float s3 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
    float s4 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3);
    float s5 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
    float t0 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
    float t1 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2);
    float t2 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
    float t3 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2);
    float t4 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
    float t5 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3);
    float det = ((s0 * t5 - s1 * t4) + (s2 * t3 + s3 * t2)) - (s4 * t1 - s5 * t0);
    float inv = 1.0f / det;
    float b[4][4];  // b[row][col] of the inverse
    b[0][0] = (a(1, 1) * t5 - a(1, 2) * t4 + a(1, 3) * t3) * inv;
    b[0][1] = (-a(0, 1) * t5 + a(0, 2) * t4 - a(0, 3) * t3) * inv;
    b[0][2] = (a(3, 1) * s5 - a(3, 2) * s4 + a(3, 3) * s3) * inv;
    b[0][3] = (-a(2, 1) * s5 + a(2, 2) * s4 - a(2, 3) * s3) * inv;
    b[1][0] = (-a(1, 0) * t5 + a(1, 2) * t2 - a(1, 3) * t1) * inv;
    b[1][1] = (a(0, 0) * t5 - a(0, 2) * t2 + a(0, 3) * t1) * inv;
    b[1][2] = (-a(3, 0) * s5 + a(3, 2) * s2 - a(3, 3) * s1) * inv;
    b[1][3] = (a(2, 0) * s5 - a(2, 2) * s2 + a(2, 3) * s1) * inv;
    b[2][0] = (a(1, 0) * t4 - a(1, 1) * t2 + a(1, 3) * t0) * inv;
    b[2][1] = (-a(0, 0) * t4 + a(0, 1) * t2 - a(0, 3) * t0) * inv;
    b[2][2] = (a(3, 0) * s4 - a(3, 1) * s2 + a(3, 3) * s0) * inv;
    b[2][3] = (-a(2, 0) * s4 + a(2, 1) * s2 - a(2, 3) * s0) * inv;
    b[3][0] = (-a(1, 0) * t3 + a(1, 1) * t1 - a(1, 2) * t0) * inv;
    b[3][1] = (a(0, 0) * t3 - a(0, 1) * t1 + a(0, 2) * t0) * inv;
    b[3][2] = (-a(3, 0) * s3 + a(3, 1) * s1 - a(3, 2) * s0) * inv;
    b[3][3] = (a(2, 0) * s3 - a(2, 1) * s1 + a(2, 2) * s0) * inv;
    mat4 r(0.0f);
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col) r[col][row] = b[row][col];
    return r;
}

// ---------------------------------------------------------------- quaternions (Hamilton)
struct quat {
    float x, y, z, w;
    constexpr quat() : x(0), y(0), z(0), w(1) {}
    constexpr quat(float w_, float x_, float y_, float z_) : x(x_), y(y_), z(z_), w(w_) {}
};
inline float dot(const quat& a, const quat& b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
inline quat operator*(const quat& p, const quat& q) {
    return quat(((p.w * q.w - p.x * q.x) - p.y * q.y) - p.z * q.z,
                ((p.w * q.x + p.x * q.w) + p.y * q.z) - p.z * q.y,
                ((p.w * q.y + p.y * q.w) + p.z * q.x) - p.x * q.z,
                ((p.w * q.z + p.z * q.w) + p.x * q.y) - p.y * q.x);
}
// Rotation of v by a unit quaternion: t = 2 (q.xyz x v); v' = v + q.w t + q.xyz x t.
inline vec3 operator*(const quat& q, const vec3& v) {
    vec3 qv(q.x, q.y, q.z);
    vec3 t = 2.0f * cross(qv, v);
    return (v + q.w * t) + cross(qv, t);
}
inline quat normalize(const quat& q) {
    float len = std::sqrt(dot(q, q));
    if (len <= 0.0f) return quat(1.0f, 0.0f, 0.0f, 0.0f);
    float inv = 1.0f / len;
    return quat(q.w * inv, q.x * inv, q.y * inv, q.z * inv);
}
inline quat conjugate(const quat& q) { return quat(q.w, -q.x, -q.y, -q.z); }
inline quat inverse(const quat& q) {
    float d = dot(q, q);
    quat c = conjugate(q);
    return quat(c.w / d, c.x / d, c.y / d, c.z / d);
}
inline quat angleAxis(float angle, const vec3& axis) {
    float s = std::sin(angle * 0.5f);
    return quat(std::cos(angle * 0.5f), axis.x * s, axis.y * s, axis.z * s);
}
// Shortest-arc rotation taking unit vector a onto unit vector b.
inline quat rotation(const vec3& a, const vec3& b) {
    float c = dot(a, b);
    if (c >= 1.0f - 1e-6f) return quat(1.0f, 0.0f, 0.0f, 0.0f);
    vec3 axis;
    if (c < -1.0f + 1e-6f) {
        axis = cross(vec3(0.0f, 0.0f, 1.0f), a);
        if (length2(axis) < 0.01f) axis = cross(vec3(1.0f, 0.0f, 0.0f), a);
        return angleAxis(pi<float>(), normalize(axis));
    }
    axis = cross(a, b);
    float s = std::sqrt((1.0f + c) * 2.0f);
    float invs = 1.0f / s;
    return quat(s * 0.5f, axis.x * invs, axis.y * invs, axis.z * invs);
}
// Rotation matrix of a unit quaternion; column j is the image of basis vector e_j.
inline mat3 mat3_cast(const quat& q) {
    float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    mat3 r;
    r[0] = vec3(1.0f - 2.0f * (yy + zz), 2.0f * (xy + wz), 2.0f * (xz - wy));
    r[1] = vec3(2.0f * (xy - wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz + wx));
    r[2] = vec3(2.0f * (xz + wy), 2.0f * (yz - wx), 1.0f - 2.0f * (xx + yy));
    return r;
}
inline mat4 mat4_cast(const quat& q) {
    mat3 m = mat3_cast(q);
    return mat4(vec4(m[0], 0.0f), vec4(m[1], 0.0f), vec4(m[2], 0.0f), vec4(0.0f, 0.0f, 0.0f, 1.0f));
}

// ---------------------------------------------------------------- transforms
// Right-handed perspective with clip z in [-w, w] (the OpenGL convention).
inline mat4 perspective(float fovy, float aspect, float zNear, float zFar) {
    float th = std::tan(fovy / 2.0f);
    mat4 r(0.0f);
    r[0][0] = 1.0f / (aspect * th);
    r[1][1] = 1.0f / th;
    r[2][2] = -(zFar + zNear) / (zFar - zNear);
    r[2][3] = -1.0f;
    r[3][2] = -((2.0f * zFar) * zNear) / (zFar - zNear);
    return r;
}
// m * T(v): column 3 becomes ((m0*v.x + m1*v.y) + m2*v.z) + m3.
inline mat4 translate(const mat4& m, const vec3& v) {
    mat4 r = m;
    r[3] = ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3];
    return r;
}
// m * R(angle, axis) with R the axis-angle rotation (Rodrigues) about normalize(axis).
inline mat4 rotate(const mat4& m, float angle, const vec3& axisIn) {
    float c = std::cos(angle), s = std::sin(angle);
    vec3 ax = normalize(axisIn);
    vec3 t = (1.0f - c) * ax;
    mat4 rot(0.0f);
    rot[0] = vec4(c + t.x * ax.x, t.x * ax.y + s * ax.z, t.x * ax.z - s * ax.y, 0.0f);
    rot[1] = vec4(t.y * ax.x - s * ax.z, c + t.y * ax.y, t.y * ax.z + s * ax.x, 0.0f);
    rot[2] = vec4(t.z * ax.x + s * ax.y, t.z * ax.y - s * ax.x, c + t.z * ax.z, 0.0f);
    rot[3] = vec4(0.0f, 0.0f, 0.0f, 1.0f);
    return m * rot;
}

inline const float* value_ptr(const mat4& m) { return &m[0].x; }
inline float* value_ptr(mat4& m) { return &m[0].x; }

}  // namespace glm
