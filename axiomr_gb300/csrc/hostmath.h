// Host float math for the per-draw uniforms and the camera helpers. Compiled with
// -ffp-contract=off; the association order of every sum is the one the kernels and the
// AxiomR math conventions use (see fmath.cuh):
//   mat4 * mat4: column j = (A0*Bj.x + A1*Bj.y) + (A2*Bj.z + A3*Bj.w)
//   dot3 = (x*x' + y*y') + z*z';  dot4 / quaternion dot = (x*x' + y*y') + (z*z' + w*w')
//   normalize(v) = v * (1 / sqrt(dot(v, v)))
#pragma once
#include <cmath>

namespace axr::host {

struct M4 {
    float m[16];  // column-major: m[4*col + row]
    float at(int row, int col) const { return m[4 * col + row]; }
};

inline M4 mul(const M4& a, const M4& b) {
    M4 r;
    for (int j = 0; j < 4; ++j) {
        const float x = b.m[4 * j], y = b.m[4 * j + 1], z = b.m[4 * j + 2], w = b.m[4 * j + 3];
        for (int i = 0; i < 4; ++i) {
            float s01 = a.m[i] * x + a.m[4 + i] * y;
            float s23 = a.m[8 + i] * z + a.m[12 + i] * w;
            r.m[4 * j + i] = s01 + s23;
        }
    }
    return r;
}

inline M4 load(const float* f) {
    M4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = f[i];
    return r;
}

inline M4 identity() {
    M4 r{};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
    return r;
}

// Inverse by the adjugate over complementary 2x2 minors (rows 0-1: s*, rows 2-3: t*):
// det = ((s0*t5 - s1*t4) + (s2*t3 + s3*t2)) - (s4*t1 - s5*t0); every adjugate entry is a
// signed three-term sum left to right, times 1/det.
inline M4 inverse(const M4& M) {
    auto a = [&](int r, int c) { return M.at(r, c); };
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
    float b[4][4];
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
    M4 r;
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col) r.m[4 * col + row] = b[row][col];
    return r;
}

// mat3(transpose(inverse(model))), column-major 3x3 (FlatShader, shaders.hpp:36-37).
inline void normal_matrix(const M4& model, float out9[9]) {
    M4 inv = inverse(model);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) out9[3 * c + r] = inv.at(c, r);
}

struct V3 {
    float x, y, z;
};
struct Q {
    float x, y, z, w;
};

inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 normalize(V3 v) {
    float s = 1.0f / std::sqrt(dot(v, v));
    return {v.x * s, v.y * s, v.z * s};
}
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float qdot(Q a, Q b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }

// Camera(position, target, fov, aspect) + update(0) (src/camera.cpp:30-100): orientation
// quaternion turning -z onto the target direction, projection perspective(radians(fov),
// aspect, 0.1, 100) with clip z in [-w, w], view = rotation(inverse(q)) * translate(-pos).
inline void camera_matrices(const float pos[3], const float target[3], float fov, float aspect, M4& view, M4& proj,
                            M4& view_proj) {
    fov = fov < 1.0f ? 1.0f : (179.0f < fov ? 179.0f : fov);
    aspect = aspect < 0.1f ? 0.1f : aspect;
    const V3 p{pos[0], pos[1], pos[2]};
    const V3 forward{0.0f, 0.0f, -1.0f};
    V3 dir = normalize({target[0] - p.x, target[1] - p.y, target[2] - p.z});
    float d = dot(forward, dir);
    auto angle_axis = [](float angle, V3 axis) {
        float s = std::sin(angle * 0.5f);
        return Q{axis.x * s, axis.y * s, axis.z * s, std::cos(angle * 0.5f)};
    };
    Q q;
    if (std::fabs(d + 1.0f) < 0.000001f) {
        q = angle_axis(3.14159265358979323846f, {0.0f, 1.0f, 0.0f});
    } else {
        V3 axis = cross(forward, dir);
        if (dot(axis, axis) < 0.000001f)
            q = Q{0.0f, 0.0f, 0.0f, 1.0f};
        else
            q = angle_axis(std::acos(d), normalize(axis));
    }
    float len = std::sqrt(qdot(q, q));
    if (len <= 0.0f) {
        q = Q{0.0f, 0.0f, 0.0f, 1.0f};
    } else {
        float inv = 1.0f / len;
        q = Q{q.x * inv, q.y * inv, q.z * inv, q.w * inv};
    }
    // projection
    float fovy = fov * 0.0174532925199432957692369076848861f;
    const float zn = 0.1f, zf = 100.0f;
    float th = std::tan(fovy / 2.0f);
    proj = M4{};
    proj.m[0] = 1.0f / (aspect * th);
    proj.m[5] = 1.0f / th;
    proj.m[10] = -(zf + zn) / (zf - zn);
    proj.m[11] = -1.0f;
    proj.m[14] = -((2.0f * zf) * zn) / (zf - zn);
    // inverse(q) = conjugate(q) / dot(q, q)
    float qq = qdot(q, q);
    Q qi{-q.x / qq, -q.y / qq, -q.z / qq, q.w / qq};
    float xx = qi.x * qi.x, yy = qi.y * qi.y, zz = qi.z * qi.z;
    float xy = qi.x * qi.y, xz = qi.x * qi.z, yz = qi.y * qi.z;
    float wx = qi.w * qi.x, wy = qi.w * qi.y, wz = qi.w * qi.z;
    M4 rot{};
    rot.m[0] = 1.0f - 2.0f * (yy + zz); rot.m[1] = 2.0f * (xy + wz); rot.m[2] = 2.0f * (xz - wy);
    rot.m[4] = 2.0f * (xy - wz); rot.m[5] = 1.0f - 2.0f * (xx + zz); rot.m[6] = 2.0f * (yz + wx);
    rot.m[8] = 2.0f * (xz + wy); rot.m[9] = 2.0f * (yz - wx); rot.m[10] = 1.0f - 2.0f * (xx + yy);
    rot.m[15] = 1.0f;
    // translate(identity, -pos): column 3 = ((I0*-x + I1*-y) + I2*-z) + I3
    M4 tr = identity();
    const float n[3] = {-p.x, -p.y, -p.z};
    for (int i = 0; i < 4; ++i) {
        const float c0 = tr.m[i], c1 = tr.m[4 + i], c2 = tr.m[8 + i], c3 = tr.m[12 + i];
        tr.m[12 + i] = ((c0 * n[0] + c1 * n[1]) + c2 * n[2]) + c3;
    }
    view = mul(rot, tr);
    view_proj = mul(proj, view);
}

// Camera::getViewportMatrix (src/camera.cpp:191-205)
inline M4 viewport_matrix(int x, int y, int w, int h) {
    M4 v = identity();
    float hw = (float)w * 0.5f, hh = (float)h * 0.5f;
    v.m[0] = hw;
    v.m[5] = -hh;
    v.m[10] = 0.5f;
    v.m[12] = (float)x + hw;
    v.m[13] = (float)y + hh;
    v.m[14] = 0.5f;
    return v;
}

}  // namespace axr::host
