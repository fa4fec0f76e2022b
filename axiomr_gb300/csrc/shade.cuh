// Texture sampling and the built-in shaders as device functors.
//
//   tex_sample        reference include/texture.hpp:12-34 (nearest, truncating
//                     x = (int)(u*(W-1)), clamp to edge, rows flipped, /255)
//   Flat              include/shaders/shaders.hpp:19-62
//   Phong             include/shaders/shaders.hpp:140-247
//   PBR               include/shaders/shaders.hpp:252-423
//   BlinnPhong        this project's shader (the reference has none): Phong's structure
//                     with the half vector H = normalize(L + V) and no normal map
//   Gouraud           this project's shader: RGB carried in Vertex::normal, A in uv.x
// Texture coordinates and barycentric interpolation use the exact-rounding helpers, so
// the texel a fragment reads is the reference's. The lighting terms after that reach the
// framebuffer only through the 8-bit quantisation: their divisions and powers use the
// colour-only helpers of fmath.cuh (relative error of a few 1e-7 on exact inputs, not
// amplified by what follows), inside the 1 LSB colour tolerance. Normalisation stays
// correctly rounded wherever the vector feeds a specular term: a sharp highlight
// (PBR's distribution term at low roughness, a large Phong exponent) would magnify a
// 1e-7 change in n.h far beyond 1 LSB. Only Flat's normal, which feeds a clamped dot
// product alone, uses the fast form. Products and sums keep the reference's order and
// rounding.
#pragma once
#include "device_types.h"
#include "fmath.cuh"
#include "raster.cuh"

namespace axr {

// A texel through the read-only path with an L2 evict_last policy: textures are shared by
// many draws and re-read across the frame, while the framebuffer planes and per-draw
// scratch stream through L2 at the default priority. The texel loads are the only reads
// that carry this policy, so L2's evict_last counters measure exactly the texture fetches.
__device__ __forceinline__ uint32_t ld_texel(const uint32_t* a) {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    uint32_t v;
    asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}

__device__ __forceinline__ f4 tex_sample(const DevTexture& t, f2 uv) {
    if (t.texels == nullptr || t.width <= 0) return mk4(0.0f, 0.0f, 0.0f, 1.0f);
    const int w = t.width, h = t.height;
    int x = __float2int_rz(fmul(uv.x, (float)(w - 1)));
    int y = __float2int_rz(fmul(uv.y, (float)(h - 1)));
    x = max(0, min(x, w - 1));
    y = max(0, min(y, h - 1));
    y = h - 1 - y;
    uint32_t p = ld_texel(&t.texels[(size_t)y * (size_t)w + (size_t)x]);
    const float inv255 = 1.0f / 255.0f;
    return mk4(fmul((float)(p & 0xFFu), inv255), fmul((float)((p >> 8) & 0xFFu), inv255),
               fmul((float)((p >> 16) & 0xFFu), inv255), fmul((float)(p >> 24), inv255));
}

// Vertex attributes a shader consumes, and the clipper attribute mask that carries them.
template <int S> struct ShaderAttrs;
template <> struct ShaderAttrs<kFlat> { static constexpr int mask = kAttrNrm; };
template <> struct ShaderAttrs<kPhong> { static constexpr int mask = kAttrPos | kAttrUv | kAttrNrm | kAttrTanBit; };
template <> struct ShaderAttrs<kPBR> { static constexpr int mask = kAttrPos | kAttrUv | kAttrNrm | kAttrTanBit; };
template <> struct ShaderAttrs<kBlinnPhong> { static constexpr int mask = kAttrPos | kAttrUv | kAttrNrm; };
template <> struct ShaderAttrs<kGouraud> { static constexpr int mask = kAttrUv | kAttrNrm; };

// VertexOutput (reference include/IShader.hpp:11-17); tbn columns are t, b, n.
struct VSOut {
    f3 normal;
    f2 uv;
    f3 world;
    f3 t, b, n;
};

template <int A>
__device__ __forceinline__ CVFull load_vertex(const DevMesh& m, uint32_t vi) {
    CVFull v;
    float4 p = __ldg(&m.pos[vi]);
    v.pos = mk3(p.x, p.y, p.z);
    if constexpr ((A & kAttrUv) != 0) {
        float2 t = __ldg(&m.uv[vi]);
        v.uv = mk2(t.x, t.y);
    }
    if constexpr ((A & kAttrNrm) != 0) {
        float4 n = __ldg(&m.nrm[vi]);
        v.nrm = mk3(n.x, n.y, n.z);
    }
    if constexpr ((A & kAttrTanBit) != 0) {
        float4 t = m.tan ? __ldg(&m.tan[vi]) : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 b = m.bit ? __ldg(&m.bit[vi]) : make_float4(0.f, 0.f, 0.f, 0.f);
        v.tan = mk3(t.x, t.y, t.z);
        v.bit = mk3(b.x, b.y, b.z);
    }
    return v;
}

__device__ __forceinline__ f3 model_dir(const DevUniforms& u, f3 d) { return xyz(mat4_mul(u.model, d.x, d.y, d.z, 0.0f)); }
__device__ __forceinline__ f3 model_point(const DevUniforms& u, f3 p) { return xyz(mat4_mul(u.model, p.x, p.y, p.z, 1.0f)); }

template <int S>
__device__ __forceinline__ VSOut vertex_shader(const DevUniforms& u, const CVFull& v) {
    VSOut o;
    if constexpr (S == kFlat) {
        o.normal = mat3_mul(u.normal_mat, v.nrm);
    } else if constexpr (S == kPhong || S == kPBR) {
        o.uv = v.uv;
        o.world = model_point(u, v.pos);
        o.t = normalize(model_dir(u, v.tan));
        o.b = normalize(model_dir(u, v.bit));
        o.n = normalize(model_dir(u, v.nrm));
    } else if constexpr (S == kBlinnPhong) {
        o.uv = v.uv;
        o.world = model_point(u, v.pos);
        o.normal = normalize(model_dir(u, v.nrm));
    } else {
        o.normal = v.nrm;
        o.uv = v.uv;
    }
    return o;
}

// Vertex-shader outputs cached per vertex (float4s per vertex) by the vertex pass:
//   Flat        [normal, 0]
//   Gouraud     [normal, uv.x]
//   BlinnPhong  [world, uv.x] [normal, uv.y]
//   Phong, PBR  [world, uv.x] [t, uv.y] [b, 0] [n, 0]
template <int S>
struct VAttr {
    static constexpr int n = vattr_float4s(S);
};
constexpr int kMaxVAttr = 4;

template <int S>
__device__ __forceinline__ void pack_vsout(const VSOut& o, float4* dst) {
    if constexpr (S == kFlat) {
        dst[0] = make_float4(o.normal.x, o.normal.y, o.normal.z, 0.0f);
    } else if constexpr (S == kGouraud) {
        dst[0] = make_float4(o.normal.x, o.normal.y, o.normal.z, o.uv.x);
    } else if constexpr (S == kBlinnPhong) {
        dst[0] = make_float4(o.world.x, o.world.y, o.world.z, o.uv.x);
        dst[1] = make_float4(o.normal.x, o.normal.y, o.normal.z, o.uv.y);
    } else {
        dst[0] = make_float4(o.world.x, o.world.y, o.world.z, o.uv.x);
        dst[1] = make_float4(o.t.x, o.t.y, o.t.z, o.uv.y);
        dst[2] = make_float4(o.b.x, o.b.y, o.b.z, 0.0f);
        dst[3] = make_float4(o.n.x, o.n.y, o.n.z, 0.0f);
    }
}

// Load of cached per-vertex data: through the read-only cache when it was written by an
// earlier launch, a plain load when it was written earlier in the same (persistent) launch.
template <bool kCoherent>
__device__ __forceinline__ float4 ld_cached(const float4* p) {
    if constexpr (kCoherent) return *p;
    else return __ldg(p);
}

template <int S, bool kCoherent = false>
__device__ __forceinline__ VSOut unpack_vsout(const float4* src) {
    VSOut o;
    if constexpr (S == kFlat) {
        float4 a = ld_cached<kCoherent>(&src[0]);
        o.normal = mk3(a.x, a.y, a.z);
    } else if constexpr (S == kGouraud) {
        float4 a = ld_cached<kCoherent>(&src[0]);
        o.normal = mk3(a.x, a.y, a.z);
        o.uv = mk2(a.w, 0.0f);
    } else if constexpr (S == kBlinnPhong) {
        float4 a = ld_cached<kCoherent>(&src[0]), b = ld_cached<kCoherent>(&src[1]);
        o.world = mk3(a.x, a.y, a.z);
        o.normal = mk3(b.x, b.y, b.z);
        o.uv = mk2(a.w, b.w);
    } else {
        float4 a = ld_cached<kCoherent>(&src[0]), b = ld_cached<kCoherent>(&src[1]), c = ld_cached<kCoherent>(&src[2]), d = ld_cached<kCoherent>(&src[3]);
        o.world = mk3(a.x, a.y, a.z);
        o.uv = mk2(a.w, b.w);
        o.t = mk3(b.x, b.y, b.z);
        o.b = mk3(c.x, c.y, c.z);
        o.n = mk3(d.x, d.y, d.z);
    }
    return o;
}

// bar.x*a + bar.y*b + bar.z*c, left to right
__device__ __forceinline__ f3 bary(f3 w, f3 a, f3 b, f3 c) { return add(add(mul(w.x, a), mul(w.y, b)), mul(w.z, c)); }
__device__ __forceinline__ f2 bary(f3 w, f2 a, f2 b, f2 c) { return add(add(mul(w.x, a), mul(w.y, b)), mul(w.z, c)); }

__device__ __forceinline__ f3 fresnel_schlick(float cos_theta, f3 f0) {
    float omc = fsub(1.0f, cos_theta);
    float term = fmul(omc, omc);
    term = fmul(term, term);
    term = fmul(term, omc);
    return add(f0, mul(sub(mk3(1.f, 1.f, 1.f), f0), term));
}

__device__ __forceinline__ f3 pow3(f3 b, f3 e) { return mk3(cpow(b.x, e.x), cpow(b.y, e.y), cpow(b.z, e.z)); }

// pow(b, e) for b = max(x, 0): pow(+0, e) is +0 for every e > 0, so that case skips the
// call (warps whose pixels all face away from the light skip it entirely).
__device__ __forceinline__ float pow_clamped(float b, float e) { return (b == 0.0f && e > 0.0f) ? 0.0f : cpow(b, e); }

template <int S>
__device__ __forceinline__ f4 fragment_shader(const DevUniforms& u, const DevMaterial& m, f3 w, const VSOut* t) {
    if constexpr (S == kFlat) {
        f3 n = cnormalize(bary(w, t[0].normal, t[1].normal, t[2].normal));
        float intensity = sclamp(dot(neg(mk3(u.light_dir[0], u.light_dir[1], u.light_dir[2])), n), 0.0f, 1.0f);
        float c = fmul(1.0f, intensity);
        return mk4(c, c, c, c);
    } else if constexpr (S == kPhong) {
        const f3 lc = mk3(u.light_color[0], u.light_color[1], u.light_color[2]);
        f2 uv = bary(w, t[0].uv, t[1].uv, t[2].uv);
        f4 nmv = tex_sample(m.bump, uv);
        f3 nms = normalize(sub(mul(xyz(nmv), 2.0f), mk3(1.f, 1.f, 1.f)));
        f3 iT = bary(w, t[0].t, t[1].t, t[2].t);
        f3 iN = normalize(bary(w, t[0].n, t[1].n, t[2].n));
        f3 iTN = normalize(sub(iT, mul(iN, dot(iN, iT))));
        f3 iBN = cross(iN, iTN);
        f4 albedo = tex_sample(m.diffuse, uv);
        f3 normal = normalize(mat3_cols_mul(iTN, iBN, iN, nms));
        f3 frag = bary(w, t[0].world, t[1].world, t[2].world);
        f3 view_dir = normalize(sub(mk3(u.cam_pos[0], u.cam_pos[1], u.cam_pos[2]), frag));
        f3 light_dir = neg(mk3(u.light_dir[0], u.light_dir[1], u.light_dir[2]));
        f3 ambient = mul(0.1f, lc);
        float diff = smax(dot(normal, light_dir), 0.0f);
        f3 diffuse = mul(diff, lc);
        f3 refl = reflect(neg(light_dir), normal);
        float spec = pow_clamped(smax(dot(view_dir, refl), 0.0f), fmul(m.specular_exponent, 50.0f));
        f3 specular = mul(fmul(0.5f, spec), lc);
        f3 c = mul(add(add(ambient, diffuse), specular), xyz(albedo));
        return mk4(c.x, c.y, c.z, 1.0f);
    } else if constexpr (S == kPBR) {
        const f3 lc = mk3(u.light_color[0], u.light_color[1], u.light_color[2]);
        const f3 one = mk3(1.f, 1.f, 1.f);
        f2 uv = bary(w, t[0].uv, t[1].uv, t[2].uv);
        f4 nmv = tex_sample(m.bump, uv);
        f3 nms = normalize(subs(mul(xyz(nmv), 2.0f), 1.0f));
        f3 c0 = bary(w, t[0].t, t[1].t, t[2].t);
        f3 c1 = bary(w, t[0].b, t[1].b, t[2].b);
        f3 c2 = bary(w, t[0].n, t[1].n, t[2].n);
        // shaders.hpp:316-322 builds a re-orthogonalised frame that nothing reads; it has
        // no effect on the colour and is not evaluated here.
        f3 albedo = pow3(xyz(tex_sample(m.diffuse, uv)), mk3(2.2f, 2.2f, 2.2f));
        float metallic = tex_sample(m.metallic, uv).x;
        float roughness = tex_sample(m.roughness, uv).x;
        float ao = tex_sample(m.ao, uv).x;
        float r2 = fmul(roughness, roughness);
        float r4 = fmul(r2, r2);
        float one_minus_metallic = fsub(1.0f, metallic);
        f3 normal = normalize(mat3_cols_mul(c0, c1, c2, nms));
        f3 frag = bary(w, t[0].world, t[1].world, t[2].world);
        f3 view_dir = normalize(sub(mk3(u.cam_pos[0], u.cam_pos[1], u.cam_pos[2]), frag));
        f3 light_dir = neg(mk3(u.light_dir[0], u.light_dir[1], u.light_dir[2]));
        f3 halfway = normalize(add(light_dir, view_dir));
        float ndoth = smax(dot(normal, halfway), 0.0f);
        float ndotv = smax(dot(normal, view_dir), 0.0f);
        float ndotl = smax(dot(normal, light_dir), 0.0f);
        const f3 f0base = mk3(0.04f, 0.04f, 0.04f);
        f3 f0 = add(f0base, mul(metallic, sub(albedo, f0base)));
        const float pi = 3.14159265358979323846f;
        float ndoth2 = fmul(ndoth, ndoth);
        float dp = fadd(fmul(ndoth2, fsub(r4, 1.0f)), 1.0f);
        float ndf = cdiv(r4, fmul(fmul(pi, dp), dp));
        float r = fadd(roughness, 1.0f);
        float k = cdiv(fmul(r, r), 8.0f);
        float nvk = fadd(fmul(ndotv, fsub(1.0f, k)), k);
        float nlk = fadd(fmul(ndotl, fsub(1.0f, k)), k);
        float g = fmul(cdiv(ndotv, nvk), cdiv(ndotl, nlk));
        f3 f = fresnel_schlick(smax(dot(halfway, normal), 0.0f), f0);
        f3 numerator = mul(mul(f, ndf), g);
        float denom = fadd(fmul(fmul(4.0f, ndotv), ndotl), 0.0001f);
        f3 specular = cdivs(numerator, denom);
        f3 kd = mul(sub(one, f), one_minus_metallic);
        f3 diffuse = mul(mul(kd, albedo), crcp(pi));
        f3 ambient = mul(mul(mk3(0.03f, 0.03f, 0.03f), albedo), ao);
        f3 c = add(ambient, mul(mul(add(diffuse, specular), lc), ndotl));
        c = cdiv(c, add(c, one));
        const float inv_gamma = 1.0f / 2.2f;
        c = pow3(c, mk3(inv_gamma, inv_gamma, inv_gamma));
        return mk4(c.x, c.y, c.z, 1.0f);
    } else if constexpr (S == kBlinnPhong) {
        const f3 lc = mk3(u.light_color[0], u.light_color[1], u.light_color[2]);
        f2 uv = bary(w, t[0].uv, t[1].uv, t[2].uv);
        f3 albedo = xyz(tex_sample(m.diffuse, uv));
        f3 n = normalize(bary(w, t[0].normal, t[1].normal, t[2].normal));
        f3 frag = bary(w, t[0].world, t[1].world, t[2].world);
        f3 view_dir = normalize(sub(mk3(u.cam_pos[0], u.cam_pos[1], u.cam_pos[2]), frag));
        f3 light_dir = neg(mk3(u.light_dir[0], u.light_dir[1], u.light_dir[2]));
        f3 halfway = normalize(add(light_dir, view_dir));
        f3 ambient = mul(0.1f, lc);
        float diff = smax(dot(n, light_dir), 0.0f);
        f3 diffuse = mul(diff, lc);
        float spec = pow_clamped(smax(dot(n, halfway), 0.0f), fmul(m.specular_exponent, 50.0f));
        f3 specular = mul(fmul(0.5f, spec), lc);
        f3 c = mul(add(add(ambient, diffuse), specular), albedo);
        return mk4(c.x, c.y, c.z, 1.0f);
    } else {
        f3 rgb = bary(w, t[0].normal, t[1].normal, t[2].normal);
        float a = fadd(fadd(fmul(w.x, t[0].uv.x), fmul(w.y, t[1].uv.x)), fmul(w.z, t[2].uv.x));
        return mk4(rgb.x, rgb.y, rgb.z, a);
    }
}

// (uint8_t)(std::clamp(c, 0, 1) * 255): truncating conversion, NaN -> 0.
// __saturatef clamps to [0, 1] and maps NaN to 0, which is the clamp followed by the NaN
// rule; the product is then in [0, 255] and truncates to the byte.
__device__ __forceinline__ uint32_t quantize(float c) {
    return (uint32_t)__float2uint_rz(fmul(__saturatef(c), 255.0f));
}

// RGBA floats -> framebuffer word with bytes B, G, R, A (reference
// src/tiled_pipeline.cpp:579-582 quantisation and 1171-1174 swizzle).
__device__ __forceinline__ uint32_t pack_bgra(f4 c) {
    return quantize(c.z) | (quantize(c.y) << 8) | (quantize(c.x) << 16) | (quantize(c.w) << 24);
}

}  // namespace axr
