// The reference Camera's state and motion on the host (src/camera.cpp:30-205,
// include/camera.hpp:6-67): construction, the setters, mouse / keyboard input and
// update(deltaTime), in the reference's float operation order. The caller owns the state
// (axr_camera_state); axr_camera_describe turns it into the axr_camera_desc that
// axr_set_camera / the batch and server descriptors take.
//
// Behaviour kept from the reference, including what looks unintended:
//   * the constructor computes the projection but leaves the view matrix at identity (and
//     viewProjection = projection) until the first update();
//   * setFov / setAspectRatio only mark the projection dirty, and nothing recomputes it
//     after the constructor, so they do not change the matrices;
//   * update() rotates only when both the yaw and the pitch delta are non-zero;
//   * the camera moves by the sum of its unit direction vectors per second (the
//     movement speed member is never used);
//   * setTarget uses the shortest-arc rotation, the constructor an angle-axis rotation.
// Quaternion products, vector rotation and the shortest-arc rotation follow the Hamilton
// conventions and sum orders of hostmath.h (dot3 left to right, quaternion dot pairwise).
#include <cmath>
#include <cstring>

#include "api_internal.h"
#include "hostmath.h"

using namespace axr::host;
using axr_internal::fail;

namespace {

constexpr float kPitchLimit = 89.0f;
constexpr float kMinDelta = 0.0001f;
constexpr float kMaxDelta = 0.5f;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kRadians = 0.0174532925199432957692369076848861f;
constexpr float kDegrees = 57.2957795130823208767981548141052f;

float fmin_glsl(float a, float b) { return (b < a) ? b : a; }
float fmax_glsl(float a, float b) { return (a < b) ? b : a; }
float clamp_glsl(float x, float lo, float hi) { return fmin_glsl(fmax_glsl(x, lo), hi); }
float clamp_std(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 scale(float s, V3 v) { return {s * v.x, s * v.y, s * v.z}; }
V3 load3(const float* f) { return {f[0], f[1], f[2]}; }
void store3(V3 v, float* f) {
    f[0] = v.x;
    f[1] = v.y;
    f[2] = v.z;
}
Q loadq(const float* f) { return {f[0], f[1], f[2], f[3]}; }
void storeq(Q q, float* f) {
    f[0] = q.x;
    f[1] = q.y;
    f[2] = q.z;
    f[3] = q.w;
}

// Hamilton product p * q
Q qmul(Q p, Q q) {
    return {((p.w * q.x + p.x * q.w) + p.y * q.z) - p.z * q.y, ((p.w * q.y + p.y * q.w) + p.z * q.x) - p.x * q.z,
            ((p.w * q.z + p.z * q.w) + p.x * q.y) - p.y * q.x, ((p.w * q.w - p.x * q.x) - p.y * q.y) - p.z * q.z};
}
// v rotated by a unit quaternion: t = 2 (q.xyz x v), v' = (v + q.w t) + q.xyz x t
V3 qrotate(Q q, V3 v) {
    const V3 qv{q.x, q.y, q.z};
    const V3 t = scale(2.0f, cross(qv, v));
    return add(add(v, scale(q.w, t)), cross(qv, t));
}
Q qnormalize(Q q) {
    const float len = std::sqrt(qdot(q, q));
    if (len <= 0.0f) return {0.0f, 0.0f, 0.0f, 1.0f};
    const float inv = 1.0f / len;
    return {q.x * inv, q.y * inv, q.z * inv, q.w * inv};
}
Q angle_axis(float angle, V3 axis) {
    const float s = std::sin(angle * 0.5f);
    return {axis.x * s, axis.y * s, axis.z * s, std::cos(angle * 0.5f)};
}
// shortest-arc rotation taking unit vector a onto unit vector b
Q shortest_arc(V3 a, V3 b) {
    const float c = dot(a, b);
    if (c >= 1.0f - 1e-6f) return {0.0f, 0.0f, 0.0f, 1.0f};
    if (c < -1.0f + 1e-6f) {
        V3 axis = cross({0.0f, 0.0f, 1.0f}, a);
        if (dot(axis, axis) < 0.01f) axis = cross({1.0f, 0.0f, 0.0f}, a);
        return angle_axis(kPi, normalize(axis));
    }
    const V3 axis = cross(a, b);
    const float s = std::sqrt((1.0f + c) * 2.0f);
    const float invs = 1.0f / s;
    return {axis.x * invs, axis.y * invs, axis.z * invs, s * 0.5f};
}

void update_vectors(axr_camera_state* c) {
    const Q q = loadq(c->orientation);
    store3(normalize(qrotate(q, {0.0f, 0.0f, -1.0f})), c->forward);
    store3(normalize(qrotate(q, {1.0f, 0.0f, 0.0f})), c->right);
    store3(normalize(qrotate(q, {0.0f, 1.0f, 0.0f})), c->up);
    c->view_dirty = 1;
}

void update_view(axr_camera_state* c) {
    if (!c->view_dirty) return;
    // mat4_cast(inverse(q)) * translate(I, -position)
    const Q q = loadq(c->orientation);
    const float qq = qdot(q, q);
    const Q qi{-q.x / qq, -q.y / qq, -q.z / qq, q.w / qq};
    const float xx = qi.x * qi.x, yy = qi.y * qi.y, zz = qi.z * qi.z;
    const float xy = qi.x * qi.y, xz = qi.x * qi.z, yz = qi.y * qi.z;
    const float wx = qi.w * qi.x, wy = qi.w * qi.y, wz = qi.w * qi.z;
    M4 rot{};
    rot.m[0] = 1.0f - 2.0f * (yy + zz); rot.m[1] = 2.0f * (xy + wz); rot.m[2] = 2.0f * (xz - wy);
    rot.m[4] = 2.0f * (xy - wz); rot.m[5] = 1.0f - 2.0f * (xx + zz); rot.m[6] = 2.0f * (yz + wx);
    rot.m[8] = 2.0f * (xz + wy); rot.m[9] = 2.0f * (yz - wx); rot.m[10] = 1.0f - 2.0f * (xx + yy);
    rot.m[15] = 1.0f;
    M4 tr = identity();
    const float n[3] = {-c->position[0], -c->position[1], -c->position[2]};
    for (int i = 0; i < 4; ++i) {
        const float c0 = tr.m[i], c1 = tr.m[4 + i], c2 = tr.m[8 + i], c3 = tr.m[12 + i];
        tr.m[12 + i] = ((c0 * n[0] + c1 * n[1]) + c2 * n[2]) + c3;
    }
    const M4 view = mul(rot, tr);
    const M4 vp = mul(load(c->projection), view);
    std::memcpy(c->view, view.m, sizeof(view.m));
    std::memcpy(c->view_proj, vp.m, sizeof(vp.m));
    c->view_dirty = 0;
}

void update_projection(axr_camera_state* c) {
    if (!c->projection_dirty) return;
    // perspective(radians(fov), aspect, near, far), clip z in [-w, w]
    const float th = std::tan((c->fov_degrees * kRadians) / 2.0f);
    const float zn = c->near_plane, zf = c->far_plane;
    M4 p{};
    p.m[0] = 1.0f / (c->aspect_ratio * th);
    p.m[5] = 1.0f / th;
    p.m[10] = -(zf + zn) / (zf - zn);
    p.m[11] = -1.0f;
    p.m[14] = -((2.0f * zf) * zn) / (zf - zn);
    const M4 vp = mul(p, load(c->view));
    std::memcpy(c->projection, p.m, sizeof(p.m));
    std::memcpy(c->view_proj, vp.m, sizeof(vp.m));
    c->projection_dirty = 0;
}

void apply_rotation(axr_camera_state* c, float yaw, float pitch) {
    const float max_speed = 45.0f * kRadians;
    yaw = clamp_glsl(yaw, -max_speed, max_speed);
    pitch = clamp_glsl(pitch, -max_speed, max_speed);
    const Q q = loadq(c->orientation);
    const Q yaw_q = angle_axis(yaw, {0.0f, 1.0f, 0.0f});
    const Q pitch_q = angle_axis(pitch, load3(c->right));
    const Q next = qmul(qmul(yaw_q, pitch_q), q);
    const V3 up = normalize(qrotate(next, {0.0f, 1.0f, 0.0f}));
    const float up_dot = dot(up, {0.0f, 1.0f, 0.0f});
    Q out;
    if (up_dot < 0.0f) {
        out = qnormalize(qmul(yaw_q, q));
    } else {
        const V3 fwd = normalize(qrotate(next, {0.0f, 0.0f, -1.0f}));
        const float deg = std::asin(clamp_glsl(fwd.y, -1.0f, 1.0f)) * kDegrees;
        out = std::fabs(deg) <= kPitchLimit ? qnormalize(next) : qnormalize(qmul(yaw_q, q));
    }
    storeq(out, c->orientation);
    update_vectors(c);
}

}  // namespace

extern "C" {

axr_status axr_camera_init(axr_camera_state* c, const float position[3], const float target[3], float fov_degrees,
                           float aspect_ratio) {
    if (!c || !position || !target) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    std::memset(c, 0, sizeof(*c));
    store3(load3(position), c->position);
    c->fov_degrees = clamp_std(fov_degrees, 1.0f, 179.0f);
    c->aspect_ratio = aspect_ratio < 0.1f ? 0.1f : aspect_ratio;
    c->near_plane = 0.1f;
    c->far_plane = 100.0f;
    c->movement_speed = 5.0f;
    c->mouse_sensitivity = 4.0f;
    c->viewport[2] = 800;
    c->viewport[3] = 600;
    c->up[1] = 1.0f;
    const M4 id = identity();
    std::memcpy(c->view, id.m, sizeof(id.m));
    std::memcpy(c->projection, id.m, sizeof(id.m));
    std::memcpy(c->view_proj, id.m, sizeof(id.m));
    c->view_dirty = 1;
    c->projection_dirty = 1;
    // orientation turning -z onto the target direction (src/camera.cpp:30-56)
    const V3 p = load3(position);
    const V3 forward{0.0f, 0.0f, -1.0f};
    const V3 dir = normalize(sub(load3(target), p));
    const float d = dot(forward, dir);
    Q q;
    if (std::fabs(d + 1.0f) < 0.000001f) {
        q = angle_axis(kPi, {0.0f, 1.0f, 0.0f});
    } else {
        const V3 axis = cross(forward, dir);
        q = dot(axis, axis) < 0.000001f ? Q{0.0f, 0.0f, 0.0f, 1.0f} : angle_axis(std::acos(d), normalize(axis));
    }
    storeq(qnormalize(q), c->orientation);
    update_vectors(c);
    update_projection(c);
    return AXR_OK;
}

axr_status axr_camera_set_position(axr_camera_state* c, const float position[3]) {
    if (!c || !position) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    store3(load3(position), c->position);
    c->view_dirty = 1;
    return AXR_OK;
}

axr_status axr_camera_set_target(axr_camera_state* c, const float target[3]) {
    if (!c || !target) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    const V3 dir = normalize(sub(load3(target), load3(c->position)));
    storeq(shortest_arc({0.0f, 0.0f, -1.0f}, dir), c->orientation);
    update_vectors(c);
    return AXR_OK;
}

axr_status axr_camera_set_fov(axr_camera_state* c, float fov_degrees) {
    if (!c) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    c->fov_degrees = clamp_std(fov_degrees, 1.0f, 179.0f);
    c->projection_dirty = 1;
    return AXR_OK;
}

axr_status axr_camera_set_aspect_ratio(axr_camera_state* c, float aspect_ratio) {
    if (!c) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    c->aspect_ratio = aspect_ratio < 0.1f ? 0.1f : aspect_ratio;
    c->projection_dirty = 1;
    return AXR_OK;
}

axr_status axr_camera_set_viewport(axr_camera_state* c, int32_t x, int32_t y, int32_t width, int32_t height) {
    if (!c) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    c->viewport[0] = x;
    c->viewport[1] = y;
    c->viewport[2] = width;
    c->viewport[3] = height;
    return AXR_OK;
}

axr_status axr_camera_handle_input(axr_camera_state* c, const axr_input_state* in) {
    if (!c || !in) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    if (in->mouse_buttons[1]) {  // right button: rotate by the mouse motion
        c->delta_yaw = -(in->mouse[0] - c->last_mouse[0]) * c->mouse_sensitivity;
        c->delta_pitch = (in->mouse[1] - c->last_mouse[1]) * c->mouse_sensitivity;
        c->view_dirty = 1;
    } else {
        c->delta_yaw = 0.0f;
        c->delta_pitch = 0.0f;
    }
    c->last_mouse[0] = in->mouse[0];
    c->last_mouse[1] = in->mouse[1];
    V3 v{0.0f, 0.0f, 0.0f};
    const V3 f = load3(c->forward), r = load3(c->right);
    if (in->keys[(unsigned char)'W']) v = add(v, f);
    if (in->keys[(unsigned char)'S']) v = sub(v, f);
    if (in->keys[(unsigned char)'A']) v = sub(v, r);
    if (in->keys[(unsigned char)'D']) v = add(v, r);
    store3(v, c->velocity);
    return AXR_OK;
}

axr_status axr_camera_update(axr_camera_state* c, float delta_time) {
    if (!c) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    if (c->delta_pitch != 0.0f && c->delta_yaw != 0.0f) {
        float yaw = (c->delta_yaw * delta_time) * kRadians;
        float pitch = (c->delta_pitch * delta_time) * kRadians;
        yaw = clamp_std(yaw, -kMaxDelta, kMaxDelta);
        pitch = clamp_std(pitch, -kMaxDelta, kMaxDelta);
        if (std::fabs(yaw) < kMinDelta) yaw = 0.0f;
        if (std::fabs(pitch) < kMinDelta) pitch = 0.0f;
        apply_rotation(c, yaw, pitch);
    }
    const V3 v = load3(c->velocity);
    if (dot(v, v) > 0.0f) {
        store3(add(load3(c->position), {v.x * delta_time, v.y * delta_time, v.z * delta_time}), c->position);
        c->view_dirty = 1;
    }
    update_view(c);
    return AXR_OK;
}

axr_status axr_camera_describe(const axr_camera_state* c, axr_camera_desc* out) {
    if (!c || !out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    std::memcpy(out->view_proj, c->view_proj, sizeof(out->view_proj));
    const M4 vpm = viewport_matrix(c->viewport[0], c->viewport[1], c->viewport[2], c->viewport[3]);
    std::memcpy(out->viewport, vpm.m, sizeof(out->viewport));
    std::memcpy(out->position, c->position, sizeof(out->position));
    return AXR_OK;
}

}  // extern "C"
