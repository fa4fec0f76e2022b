// Device float math with explicit IEEE rounding.
//
// Coverage, depth-test winners and texture coordinates must match AxiomR's CPU pipeline
// bit for bit, so every multiply, add, divide and square root on those paths is a
// separately rounded IEEE operation (the __f*_rn intrinsics are never contracted into
// FMA), in the association order AxiomR's math library evaluates:
//   dot3 = (a.x*b.x + a.y*b.y) + a.z*b.z
//   mat3 * v = (c0*v.x + c1*v.y) + c2*v.z
//   mat4 * v = (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w)
//   normalize(v) = v * (1 / sqrt(dot(v, v)))
//   mix(x, y, a) = x*(1-a) + y*a
// (reference call sites: src/tiled_pipeline.cpp:210-212, src/pipeline.cpp:252-269,
// include/shaders/shaders.hpp). The library is additionally built with --fmad=false.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_types.h"

namespace axr {

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
// 1/x correctly rounded: the same bits as the IEEE division 1.0f / x.
__device__ __forceinline__ float frcp(float a) { return __frcp_rn(a); }
// std::max / std::min / std::clamp comparison semantics (NaN follows operator<)
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float sclamp(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

__device__ __forceinline__ f2 mk2(float x, float y) { return {x, y}; }
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f4 mk4(float x, float y, float z, float w) { return {x, y, z, w}; }
__device__ __forceinline__ f3 xyz(f4 a) { return {a.x, a.y, a.z}; }

__device__ __forceinline__ f2 add(f2 a, f2 b) { return {fadd(a.x, b.x), fadd(a.y, b.y)}; }
__device__ __forceinline__ f2 mul(f2 a, float s) { return {fmul(a.x, s), fmul(a.y, s)}; }
__device__ __forceinline__ f2 mul(float s, f2 a) { return {fmul(s, a.x), fmul(s, a.y)}; }
__device__ __forceinline__ f2 divs(f2 a, float s) { return {fdiv(a.x, s), fdiv(a.y, s)}; }

__device__ __forceinline__ f3 add(f3 a, f3 b) { return {fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)}; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return {fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)}; }
__device__ __forceinline__ f3 mul(f3 a, f3 b) { return {fmul(a.x, b.x), fmul(a.y, b.y), fmul(a.z, b.z)}; }
__device__ __forceinline__ f3 div(f3 a, f3 b) { return {fdiv(a.x, b.x), fdiv(a.y, b.y), fdiv(a.z, b.z)}; }
__device__ __forceinline__ f3 mul(f3 a, float s) { return {fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)}; }
__device__ __forceinline__ f3 mul(float s, f3 a) { return {fmul(s, a.x), fmul(s, a.y), fmul(s, a.z)}; }
__device__ __forceinline__ f3 divs(f3 a, float s) { return {fdiv(a.x, s), fdiv(a.y, s), fdiv(a.z, s)}; }
__device__ __forceinline__ f3 subs(f3 a, float s) { return {fsub(a.x, s), fsub(a.y, s), fsub(a.z, s)}; }
__device__ __forceinline__ f3 neg(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z)); }
__device__ __forceinline__ f3 normalize(f3 v) { return mul(v, frcp(fsqrt(dot(v, v)))); }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
            fsub(fmul(a.x, b.y), fmul(a.y, b.x))};
}
__device__ __forceinline__ f3 mix(f3 x, f3 y, float a) { return add(mul(x, fsub(1.0f, a)), mul(y, a)); }
__device__ __forceinline__ f2 mix(f2 x, f2 y, float a) { return add(mul(x, fsub(1.0f, a)), mul(y, a)); }
__device__ __forceinline__ float mix(float x, float y, float a) { return fadd(fmul(x, fsub(1.0f, a)), fmul(y, a)); }
__device__ __forceinline__ f3 reflect(f3 i, f3 n) { return sub(i, mul(fmul(2.0f, dot(n, i)), n)); }

__device__ __forceinline__ f4 add(f4 a, f4 b) {
    return {fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z), fadd(a.w, b.w)};
}
__device__ __forceinline__ f4 mul(f4 a, float s) { return {fmul(a.x, s), fmul(a.y, s), fmul(a.z, s), fmul(a.w, s)}; }
__device__ __forceinline__ f4 mix(f4 x, f4 y, float a) { return add(mul(x, fsub(1.0f, a)), mul(y, a)); }

// Colour-only math: for lighting terms that reach the framebuffer only through the 8-bit
// quantisation (never coverage, depth or a texture coordinate). Each result carries a
// relative error of a few 1e-7 at most, far inside the 1 LSB colour tolerance, at a
// fraction of the cost of the correctly rounded sequences:
//   crcp(x)        rcp.approx.f32 (max 1 ulp over the full range, subnormals kept):
//                  0 -> inf, inf -> 0, NaN -> NaN, as 1/x
//   cdiv(a, b)     a * crcp(b): the IEEE special cases of a/b (0/0, inf/inf -> NaN)
//   cnormalize(v)  v * rsqrtf(v.v): scales v without turning it, so the direction is the
//                  exact one; zero vectors give NaN as 1/sqrt(0) does
//   cpow(b, e)     exp2f(e * log2f(b)) for b >= 0: relative error about
//                  ln2 * |e log2 b| * 2^-23 + 2 ulp, which stays near 1e-6 wherever the
//                  power is large enough to move an 8-bit channel, for any exponent;
//                  as powf: e = 0 or b = 1 gives 1, b = 0 gives 0 (e > 0) or inf
//                  (e < 0), b < 0 (non-integer e) or NaN gives NaN
__device__ __forceinline__ float crcp(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float cdiv(float a, float b) { return fmul(a, crcp(b)); }
__device__ __forceinline__ f3 cdiv(f3 a, f3 b) { return {cdiv(a.x, b.x), cdiv(a.y, b.y), cdiv(a.z, b.z)}; }
__device__ __forceinline__ f3 cdivs(f3 a, float s) { return mul(a, crcp(s)); }
__device__ __forceinline__ f3 cnormalize(f3 v) { return mul(v, rsqrtf(dot(v, v))); }
__device__ __forceinline__ float cpow(float b, float e) {
    return (e == 0.0f || b == 1.0f) ? 1.0f : exp2f(fmul(e, log2f(b)));
}

// Column-major 4x4 (m[4*col + row]) times (x, y, z, w): pairwise sum of the four columns.
__device__ __forceinline__ f4 mat4_mul(const float* m, float x, float y, float z, float w) {
    f4 c0 = mk4(m[0], m[1], m[2], m[3]), c1 = mk4(m[4], m[5], m[6], m[7]);
    f4 c2 = mk4(m[8], m[9], m[10], m[11]), c3 = mk4(m[12], m[13], m[14], m[15]);
    return add(add(mul(c0, x), mul(c1, y)), add(mul(c2, z), mul(c3, w)));
}
// Column-major 3x3 (m[3*col + row]) times v: left-to-right sum of the three columns.
__device__ __forceinline__ f3 mat3_mul(const float* m, f3 v) {
    f3 c0 = mk3(m[0], m[1], m[2]), c1 = mk3(m[3], m[4], m[5]), c2 = mk3(m[6], m[7], m[8]);
    return add(add(mul(c0, v.x), mul(c1, v.y)), mul(c2, v.z));
}
__device__ __forceinline__ f3 mat3_cols_mul(f3 c0, f3 c1, f3 c2, f3 v) {
    return add(add(mul(c0, v.x), mul(c1, v.y)), mul(c2, v.z));
}

// Depth keys: a 64-bit value whose unsigned order is (depth, draw order). The high word
// maps the float depth to an unsigned integer with the same order (-0 folded onto +0,
// since the reference's '<' treats them as equal); the low word is the triangle's
// position in draw order, so ties go to the earliest triangle as with the reference's
// sequential strict less-than early-Z.
__device__ __forceinline__ uint32_t depth_order_bits(float z) {
    uint32_t u = __float_as_uint(z);
    if ((u << 1) == 0u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long make_key(float z, uint32_t tag) {
    return ((unsigned long long)depth_order_bits(z) << 32) | tag;
}

}  // namespace axr
