/* Oracle test infrastructure: texture sampling and the shaders, restating reference
 * include/texture.hpp:12-34 (Texture::sample) and include/shaders/shaders.hpp
 * (FlatShader 19-62, PhongShader 140-247, PBRShader 252-423), plus this project's
 * Blinn-Phong and Gouraud shaders (the reference ships neither; they follow PhongShader's
 * structure and are defined identically in oracle/ref_harness.cpp). */
#include <string.h>

#include "axo_port.h"

/* texture.hpp:12-34: nearest texel, x = (int)(u*(W-1)) truncating, clamp to edge,
 * rows flipped (y = H-1-y), channels scaled by 1/255. No data -> (0,0,0,1). */
v4 port_tex_sample(const axo_texture* t, v2 uv) {
    if (!t || !t->rgba || t->width <= 0) return V4(0.0f, 0.0f, 0.0f, 1.0f);
    int w = t->width, h = t->height;
    int x = (int)(uv.x * (float)(w - 1));
    int y = (int)(uv.y * (float)(h - 1));
    x = x < (w - 1) ? x : (w - 1);
    x = x > 0 ? x : 0;
    y = y < (h - 1) ? y : (h - 1);
    y = y > 0 ? y : 0;
    y = h - 1 - y;
    const uint8_t* p = t->rgba + ((size_t)y * (size_t)w + (size_t)x) * 4;
    const float inv255 = 1.0f / 255.0f;
    return V4((float)p[0] * inv255, (float)p[1] * inv255, (float)p[2] * inv255, (float)p[3] * inv255);
}

void shader_init(shader_state* s, const axo_shader* sh, const m4* model, const m4* view_proj, v3 cam_pos) {
    memset(s, 0, sizeof(*s));
    s->kind = sh->kind;
    s->light_dir = V3(sh->light_direction[0], sh->light_direction[1], sh->light_direction[2]);
    s->light_color = V3(sh->light_color[0], sh->light_color[1], sh->light_color[2]);
    s->model = *model;
    s->view_proj = *view_proj;
    s->mvp = m4m(view_proj, model); /* tiled_pipeline.cpp:149 */
    s->cam_pos = cam_pos;
    /* FlatShader: mat3(transpose(inverse(model))) (shaders.hpp:36-37); the reference
     * recomputes it per vertex, the value is the same every time. */
    m4 inv = m4_inverse(model);
    /* transpose: column c of transpose(inv) is row c of inv */
    for (int c = 0; c < 3; ++c) s->normal_mat.c[c] = V3(m4_at(&inv, c, 0), m4_at(&inv, c, 1), m4_at(&inv, c, 2));
}

static v3 model_dir(const shader_state* s, v3 d) { return xyz(m4v(&s->model, V4(d.x, d.y, d.z, 0.0f))); }

vsout shader_vertex(const shader_state* s, const cvert* v) {
    vsout o;
    memset(&o, 0, sizeof(o));
    switch (s->kind) {
        case AXO_FLAT: /* shaders.hpp:26-40 */
            o.normal = m3v(&s->normal_mat, v->nrm);
            break;
        case AXO_PHONG: /* shaders.hpp:147-168 */
        case AXO_PBR:   /* shaders.hpp:259-282 */
            o.uv = v->uv;
            o.world = xyz(m4v(&s->model, V4(v->pos.x, v->pos.y, v->pos.z, 1.0f)));
            o.tbn[0] = normalize3(model_dir(s, v->tan));
            o.tbn[1] = normalize3(model_dir(s, v->bit));
            o.tbn[2] = normalize3(model_dir(s, v->nrm));
            break;
        case AXO_BLINN_PHONG:
            o.uv = v->uv;
            o.world = xyz(m4v(&s->model, V4(v->pos.x, v->pos.y, v->pos.z, 1.0f)));
            o.normal = normalize3(model_dir(s, v->nrm));
            break;
        case AXO_GOURAUD:
            o.normal = v->nrm;
            o.uv = v->uv;
            break;
        default: break;
    }
    return o;
}

/* bar.x*a + bar.y*b + bar.z*c, left to right */
static v3 bary3(v3 bar, v3 a, v3 b, v3 c) { return add3(add3(smul3(bar.x, a), smul3(bar.y, b)), smul3(bar.z, c)); }
static v2 bary2(v3 bar, v2 a, v2 b, v2 c) { return add2(add2(smul2(bar.x, a), smul2(bar.y, b)), smul2(bar.z, c)); }

static v4 frag_flat(const shader_state* s, v3 bar, const vsout* t) {
    v3 n = normalize3(bary3(bar, t[0].normal, t[1].normal, t[2].normal));
    float intensity = clampf_std(dot3(neg3(s->light_dir), n), 0.0f, 1.0f);
    return V4(1.0f * intensity, 1.0f * intensity, 1.0f * intensity, 1.0f * intensity);
}

static v4 frag_phong(const shader_state* s, const axo_material* m, v3 bar, const vsout* t) {
    v2 uv = bary2(bar, t[0].uv, t[1].uv, t[2].uv);
    v4 nmv = port_tex_sample(&m->bump, uv);
    v3 nms = normalize3(sub3(mul3s(xyz(nmv), 2.0f), V3(1.0f, 1.0f, 1.0f)));
    v3 iT = bary3(bar, t[0].tbn[0], t[1].tbn[0], t[2].tbn[0]);
    v3 iN = bary3(bar, t[0].tbn[2], t[1].tbn[2], t[2].tbn[2]);
    iN = normalize3(iN);
    v3 iTN = normalize3(sub3(iT, mul3s(iN, dot3(iN, iT))));
    v3 iBN = cross3(iN, iTN);
    m3 fin;
    fin.c[0] = iTN; fin.c[1] = iBN; fin.c[2] = iN;
    v4 albedo = port_tex_sample(&m->diffuse, uv);
    v3 normal = normalize3(m3v(&fin, nms));
    v3 frag_pos = bary3(bar, t[0].world, t[1].world, t[2].world);
    v3 view_dir = normalize3(sub3(s->cam_pos, frag_pos));
    v3 light_dir = neg3(s->light_dir);
    v3 ambient = smul3(0.1f, s->light_color);
    float diff = maxf_std(dot3(normal, light_dir), 0.0f);
    v3 diffuse = smul3(diff, s->light_color);
    v3 reflect_dir = reflect3(neg3(light_dir), normal);
    float spec = powf(maxf_std(dot3(view_dir, reflect_dir), 0.0f), m->specular_exponent * 50.0f);
    v3 specular = smul3(0.5f * spec, s->light_color);
    v3 c = mul3(add3(add3(ambient, diffuse), specular), xyz(albedo));
    return V4(c.x, c.y, c.z, 1.0f);
}

static v3 fresnel_schlick(float cos_theta, v3 f0) {
    float omc = 1.0f - cos_theta;
    float term = omc * omc;
    term *= term;
    term *= omc;
    return add3(f0, mul3s(sub3(V3(1.0f, 1.0f, 1.0f), f0), term));
}

static v4 frag_pbr(const shader_state* s, const axo_material* m, v3 bar, const vsout* t) {
    v2 uv = bary2(bar, t[0].uv, t[1].uv, t[2].uv);
    v4 nmv = port_tex_sample(&m->bump, uv);
    v3 nms = normalize3(sub3s(mul3s(xyz(nmv), 2.0f), 1.0f));
    m3 itbn;
    for (int k = 0; k < 3; ++k) itbn.c[k] = bary3(bar, t[0].tbn[k], t[1].tbn[k], t[2].tbn[k]);
    /* shaders.hpp:316-322: re-orthogonalised frame, computed but not used below */
    v3 iT = itbn.c[0];
    v3 iN = normalize3(itbn.c[2]);
    v3 nt = mul3s(iN, dot3(iN, iT));
    v3 iTN = normalize3(sub3(iT, nt));
    v3 iBN = normalize3(cross3(iN, iTN));
    iN = normalize3(cross3(iTN, iBN));
    (void)iN;
    v3 albedo = xyz(port_tex_sample(&m->diffuse, uv));
    albedo = pow3(albedo, V3(2.2f, 2.2f, 2.2f));
    float metallic = port_tex_sample(&m->metallic, uv).x;
    float roughness = port_tex_sample(&m->roughness, uv).x;
    float ao = port_tex_sample(&m->ao, uv).x;
    float r2 = roughness * roughness;
    float r4 = r2 * r2;
    float one_minus_metallic = 1.0f - metallic;
    v3 normal = normalize3(m3v(&itbn, nms)); /* shaders.hpp:343 uses the interpolated TBN */
    v3 frag_pos = bary3(bar, t[0].world, t[1].world, t[2].world);
    v3 view_dir = normalize3(sub3(s->cam_pos, frag_pos));
    v3 light_dir = neg3(s->light_dir);
    v3 halfway = normalize3(add3(light_dir, view_dir));
    float ndoth = maxf_std(dot3(normal, halfway), 0.0f);
    float ndotv = maxf_std(dot3(normal, view_dir), 0.0f);
    float ndotl = maxf_std(dot3(normal, light_dir), 0.0f);
    v3 f0base = V3(0.04f, 0.04f, 0.04f);
    v3 f0 = add3(f0base, smul3(metallic, sub3(albedo, f0base))); /* lerp: a + t*(b-a) */
    const float pi = 3.14159265358979323846f;
    float ndoth2 = ndoth * ndoth;
    float dp = ndoth2 * (r4 - 1.0f) + 1.0f;
    float ndf = r4 / (pi * dp * dp);
    float r = roughness + 1.0f;
    float k = (r * r) / 8.0f;
    float nvk = ndotv * (1.0f - k) + k;
    float nlk = ndotl * (1.0f - k) + k;
    float g = (ndotv / nvk) * (ndotl / nlk);
    v3 f = fresnel_schlick(maxf_std(dot3(halfway, normal), 0.0f), f0);
    v3 numerator = mul3s(mul3s(f, ndf), g);
    float denom = 4.0f * ndotv * ndotl + 0.0001f;
    v3 specular = div3s(numerator, denom);
    v3 kd = mul3s(sub3(V3(1.0f, 1.0f, 1.0f), f), one_minus_metallic);
    v3 diffuse = mul3s(mul3(kd, albedo), 1.0f / pi);
    v3 ambient = mul3s(mul3(V3(0.03f, 0.03f, 0.03f), albedo), ao);
    v3 c = add3(ambient, mul3s(mul3(add3(diffuse, specular), s->light_color), ndotl));
    c = div3(c, add3(c, V3(1.0f, 1.0f, 1.0f)));
    c = pow3(c, V3(1.0f / 2.2f, 1.0f / 2.2f, 1.0f / 2.2f));
    return V4(c.x, c.y, c.z, 1.0f);
}

static v4 frag_blinn_phong(const shader_state* s, const axo_material* m, v3 bar, const vsout* t) {
    v2 uv = bary2(bar, t[0].uv, t[1].uv, t[2].uv);
    v3 albedo = xyz(port_tex_sample(&m->diffuse, uv));
    v3 n = normalize3(bary3(bar, t[0].normal, t[1].normal, t[2].normal));
    v3 frag_pos = bary3(bar, t[0].world, t[1].world, t[2].world);
    v3 view_dir = normalize3(sub3(s->cam_pos, frag_pos));
    v3 light_dir = neg3(s->light_dir);
    v3 halfway = normalize3(add3(light_dir, view_dir));
    v3 ambient = smul3(0.1f, s->light_color);
    float diff = maxf_std(dot3(n, light_dir), 0.0f);
    v3 diffuse = smul3(diff, s->light_color);
    float spec = powf(maxf_std(dot3(n, halfway), 0.0f), m->specular_exponent * 50.0f);
    v3 specular = smul3(0.5f * spec, s->light_color);
    v3 c = mul3(add3(add3(ambient, diffuse), specular), albedo);
    return V4(c.x, c.y, c.z, 1.0f);
}

static v4 frag_gouraud(v3 bar, const vsout* t) {
    v3 rgb = bary3(bar, t[0].normal, t[1].normal, t[2].normal);
    float a = (bar.x * t[0].uv.x + bar.y * t[1].uv.x) + bar.z * t[2].uv.x;
    return V4(rgb.x, rgb.y, rgb.z, a);
}

v4 shader_fragment(const shader_state* s, const axo_material* m, v3 bar, const vsout tri[3]) {
    switch (s->kind) {
        case AXO_FLAT: return frag_flat(s, bar, tri);
        case AXO_PHONG: return frag_phong(s, m, bar, tri);
        case AXO_PBR: return frag_pbr(s, m, bar, tri);
        case AXO_BLINN_PHONG: return frag_blinn_phong(s, m, bar, tri);
        case AXO_GOURAUD: return frag_gouraud(bar, tri);
        default: return V4(0, 0, 0, 0);
    }
}

int port_sample(const axo_texture* t, const float* uv, int n, float* out) {
    if (!t || !t->rgba || t->width <= 0) return 1;
    for (int i = 0; i < n; ++i) {
        v4 c = port_tex_sample(t, V2(uv[2 * i], uv[2 * i + 1]));
        out[4 * i] = c.x; out[4 * i + 1] = c.y; out[4 * i + 2] = c.z; out[4 * i + 3] = c.w;
    }
    return 0;
}

int port_shade(const axo_shader* sh, const axo_material* mat, const float* model, const float* view_proj,
               const float* cam_pos, const float* verts, const float* bar, float* out) {
    if (sh->kind < AXO_FLAT || sh->kind > AXO_GOURAUD) return 1;
    m4 m = m4_load(model), vp = m4_load(view_proj);
    shader_state s;
    shader_init(&s, sh, &m, &vp, V3(cam_pos[0], cam_pos[1], cam_pos[2]));
    vsout t[3];
    for (int k = 0; k < 3; ++k) {
        const float* f = verts + 14 * k;
        cvert v;
        memset(&v, 0, sizeof(v));
        v.pos = V3(f[0], f[1], f[2]);
        v.uv = V2(f[3], f[4]);
        v.nrm = V3(f[5], f[6], f[7]);
        v.tan = V3(f[8], f[9], f[10]);
        v.bit = V3(f[11], f[12], f[13]);
        t[k] = shader_vertex(&s, &v);
    }
    v4 c = shader_fragment(&s, mat, V3(bar[0], bar[1], bar[2]), t);
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
    return 0;
}
