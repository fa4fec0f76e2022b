/* Oracle test infrastructure: 4x4 inverse in the order oracle/shim/glm/glm.hpp documents
 * (adjugate over complementary 2x2 minors, scaled by 1/det). */
#include "vmath.h"

m4 m4_inverse(const m4* m) {
#define A(r, c) m4_at(m, r, c)
    float s0 = A(0, 0) * A(1, 1) - A(1, 0) * A(0, 1);
    float s1 = A(0, 0) * A(1, 2) - A(1, 0) * A(0, 2);
    float s2 = A(0, 0) * A(1, 3) - A(1, 0) * A(0, 3);
    float s3 = A(0, 1) * A(1, 2) - A(1, 1) * A(0, 2);
    float s4 = A(0, 1) * A(1, 3) - A(1, 1) * A(0, 3);
    float s5 = A(0, 2) * A(1, 3) - A(1, 2) * A(0, 3);
    float t0 = A(2, 0) * A(3, 1) - A(3, 0) * A(2, 1);
    float t1 = A(2, 0) * A(3, 2) - A(3, 0) * A(2, 2);
    float t2 = A(2, 0) * A(3, 3) - A(3, 0) * A(2, 3);
    float t3 = A(2, 1) * A(3, 2) - A(3, 1) * A(2, 2);
    float t4 = A(2, 1) * A(3, 3) - A(3, 1) * A(2, 3);
    float t5 = A(2, 2) * A(3, 3) - A(3, 2) * A(2, 3);
    float det = ((s0 * t5 - s1 * t4) + (s2 * t3 + s3 * t2)) - (s4 * t1 - s5 * t0);
    float inv = 1.0f / det;
    float b[4][4];
    b[0][0] = (A(1, 1) * t5 - A(1, 2) * t4 + A(1, 3) * t3) * inv;
    b[0][1] = (-A(0, 1) * t5 + A(0, 2) * t4 - A(0, 3) * t3) * inv;
    b[0][2] = (A(3, 1) * s5 - A(3, 2) * s4 + A(3, 3) * s3) * inv;
    b[0][3] = (-A(2, 1) * s5 + A(2, 2) * s4 - A(2, 3) * s3) * inv;
    b[1][0] = (-A(1, 0) * t5 + A(1, 2) * t2 - A(1, 3) * t1) * inv;
    b[1][1] = (A(0, 0) * t5 - A(0, 2) * t2 + A(0, 3) * t1) * inv;
    b[1][2] = (-A(3, 0) * s5 + A(3, 2) * s2 - A(3, 3) * s1) * inv;
    b[1][3] = (A(2, 0) * s5 - A(2, 2) * s2 + A(2, 3) * s1) * inv;
    b[2][0] = (A(1, 0) * t4 - A(1, 1) * t2 + A(1, 3) * t0) * inv;
    b[2][1] = (-A(0, 0) * t4 + A(0, 1) * t2 - A(0, 3) * t0) * inv;
    b[2][2] = (A(3, 0) * s4 - A(3, 1) * s2 + A(3, 3) * s0) * inv;
    b[2][3] = (-A(2, 0) * s4 + A(2, 1) * s2 - A(2, 3) * s0) * inv;
    b[3][0] = (-A(1, 0) * t3 + A(1, 1) * t1 - A(1, 2) * t0) * inv;
    b[3][1] = (A(0, 0) * t3 - A(0, 1) * t1 + A(0, 2) * t0) * inv;
    b[3][2] = (-A(3, 0) * s3 + A(3, 1) * s1 - A(3, 2) * s0) * inv;
    b[3][3] = (A(2, 0) * s3 - A(2, 1) * s1 + A(2, 2) * s0) * inv;
#undef A
    m4 r;
    for (int col = 0; col < 4; ++col) r.c[col] = V4(b[0][col], b[1][col], b[2][col], b[3][col]);
    return r;
}
