/* Oracle test infrastructure: camera matrices, restating reference src/camera.cpp:30-100
 * (constructor, updateProjectionMatrix, update(0) -> updateViewMatrix) with the
 * operation order of the oracle's glm-compatible header. */
#include "axo_port.h"

typedef struct { float x, y, z, w; } quat;

static float qdot(quat a, quat b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }

/* angleAxis: (cos(a/2), axis * sin(a/2)) */
static quat angle_axis(float angle, v3 axis) {
    float s = sinf(angle * 0.5f);
    quat q = {axis.x * s, axis.y * s, axis.z * s, cosf(angle * 0.5f)};
    return q;
}

static quat qnormalize(quat q) {
    float len = sqrtf(qdot(q, q));
    if (len <= 0.0f) { quat id = {0, 0, 0, 1}; return id; }
    float inv = 1.0f / len;
    quat r = {q.x * inv, q.y * inv, q.z * inv, q.w * inv};
    return r;
}

static quat qinverse(quat q) {
    float d = qdot(q, q);
    quat r = {-q.x / d, -q.y / d, -q.z / d, q.w / d};
    return r;
}

static m4 mat4_cast(quat q) {
    float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    m4 r;
    r.c[0] = V4(1.0f - 2.0f * (yy + zz), 2.0f * (xy + wz), 2.0f * (xz - wy), 0.0f);
    r.c[1] = V4(2.0f * (xy - wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz + wx), 0.0f);
    r.c[2] = V4(2.0f * (xz + wy), 2.0f * (yz - wx), 1.0f - 2.0f * (xx + yy), 0.0f);
    r.c[3] = V4(0.0f, 0.0f, 0.0f, 1.0f);
    return r;
}

static m4 identity(void) {
    m4 r;
    r.c[0] = V4(1, 0, 0, 0); r.c[1] = V4(0, 1, 0, 0); r.c[2] = V4(0, 0, 1, 0); r.c[3] = V4(0, 0, 0, 1);
    return r;
}

void port_camera_matrices(const axo_camera* c, m4* view, m4* proj, m4* view_proj) {
    v3 pos = V3(c->position[0], c->position[1], c->position[2]);
    v3 target = V3(c->target[0], c->target[1], c->target[2]);
    float fov = clampf_std(c->fov_degrees, 1.0f, 179.0f);  /* camera.cpp:13-15 */
    float aspect = maxf_std(c->aspect, 0.1f);               /* camera.cpp:17-19 */
    /* constructor, camera.cpp:30-56 */
    v3 forward = V3(0.0f, 0.0f, -1.0f);
    v3 direction = normalize3(sub3(target, pos));
    float d = dot3(forward, direction);
    quat q;
    if (fabsf(d + 1.0f) < 0.000001f) {
        q = angle_axis(3.14159265358979323846f, V3(0.0f, 1.0f, 0.0f));
    } else {
        v3 axis = cross3(forward, direction);
        if (dot3(axis, axis) < 0.000001f) {
            quat id = {0, 0, 0, 1};
            q = id;
        } else {
            q = angle_axis(acosf(d), normalize3(axis));
        }
    }
    q = qnormalize(q);
    /* updateProjectionMatrix, camera.cpp:75-81: perspective(radians(fov), aspect, 0.1, 100) */
    float fovy = fov * 0.0174532925199432957692369076848861f;
    float zn = 0.1f, zf = 100.0f;
    float th = tanf(fovy / 2.0f);
    m4 p;
    for (int j = 0; j < 4; ++j) p.c[j] = V4(0, 0, 0, 0);
    p.c[0].x = 1.0f / (aspect * th);
    p.c[1].y = 1.0f / th;
    p.c[2].z = -(zf + zn) / (zf - zn);
    p.c[2].w = -1.0f;
    p.c[3].z = -((2.0f * zf) * zn) / (zf - zn);
    /* update(0) -> updateViewMatrix, camera.cpp:65-73: mat4_cast(inverse(q)) * translate(I, -pos) */
    m4 rot = mat4_cast(qinverse(q));
    m4 id = identity();
    v3 np = neg3(pos);
    m4 tr = id;
    tr.c[3] = add4(add4(add4(mul4s(id.c[0], np.x), mul4s(id.c[1], np.y)), mul4s(id.c[2], np.z)), id.c[3]);
    *view = m4m(&rot, &tr);
    *proj = p;
    *view_proj = m4m(&p, view);
}

int port_camera(const axo_camera* c, float* out48) {
    m4 v, p, vp;
    port_camera_matrices(c, &v, &p, &vp);
    m4_store(&v, out48);
    m4_store(&p, out48 + 16);
    m4_store(&vp, out48 + 32);
    return 0;
}
