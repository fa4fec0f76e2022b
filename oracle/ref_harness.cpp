// Oracle test infrastructure: drives the AxiomR reference sources, compiled unmodified
// from the reference tree by oracle/build.py into oracle/_ref/libaxr_ref.so, from flat
// arrays. Used here (x86) to pin the C restatement in oracle/port and to generate the
// golden fixtures under tests/golden. The product never links or loads it.
//
// Entry points mirror oracle/port/axo_port.h one for one (ref_* vs port_*).
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fcntl.h>
#include <memory>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

#include "camera.hpp"
#include "framebuffer.hpp"
#include "mesh.hpp"
#include "shaders/shaders.hpp"
#include "texture.hpp"
#include "tiled_pipeline.hpp"
#include "window.hpp"

#include "axo.h"

namespace {

// Standard-conforming access to private data members: explicit template instantiation
// may name private members, and the friend function exports the member pointer.
template <typename Tag, typename Tag::type M>
struct Expose {
    friend typename Tag::type member(Tag) { return M; }
};
struct MeshVertices { using type = std::vector<AR::Vertex> AR::Mesh::*; friend type member(MeshVertices); };
struct MeshFaces { using type = std::vector<AR::Face> AR::Mesh::*; friend type member(MeshFaces); };
struct MeshMaterials {
    using type = std::unordered_map<std::string, std::unique_ptr<AR::Material>> AR::Mesh::*;
    friend type member(MeshMaterials);
};
struct MeshGroups { using type = std::vector<AR::MaterialGroup> AR::Mesh::*; friend type member(MeshGroups); };
struct TexData { using type = unsigned char* AR::Texture::*; friend type member(TexData); };
struct TexWidth { using type = int AR::Texture::*; friend type member(TexWidth); };
struct TexHeight { using type = int AR::Texture::*; friend type member(TexHeight); };
struct TexChannels { using type = int AR::Texture::*; friend type member(TexChannels); };
struct CamViewProj { using type = glm::mat4 AR::Camera::*; friend type member(CamViewProj); };
struct CamPosition { using type = glm::vec3 AR::Camera::*; friend type member(CamPosition); };
struct WinMouse { using type = glm::vec2 AR::Window::*; friend type member(WinMouse); };
struct WinButtons { using type = bool (AR::Window::*)[3]; friend type member(WinButtons); };
struct WinKeys { using type = bool (AR::Window::*)[256]; friend type member(WinKeys); };
template struct Expose<MeshVertices, &AR::Mesh::m_Vertices>;
template struct Expose<MeshFaces, &AR::Mesh::m_Faces>;
template struct Expose<MeshMaterials, &AR::Mesh::m_Materials>;
template struct Expose<MeshGroups, &AR::Mesh::m_MaterialGroups>;
template struct Expose<TexData, &AR::Texture::m_Data>;
template struct Expose<TexWidth, &AR::Texture::m_Width>;
template struct Expose<TexHeight, &AR::Texture::m_Height>;
template struct Expose<TexChannels, &AR::Texture::m_Channels>;
template struct Expose<CamViewProj, &AR::Camera::m_ViewProjection>;
template struct Expose<CamPosition, &AR::Camera::m_Position>;
template struct Expose<WinMouse, &AR::Window::m_MousePos>;
template struct Expose<WinButtons, &AR::Window::m_MouseButtons>;
template struct Expose<WinKeys, &AR::Window::m_Keys>;

// Pipeline::clipTriangle is protected static (reference include/pipeline.hpp:34-42).
struct ClipAccess : AR::Pipeline {
    using AR::Pipeline::clipTriangle;
};

// Shader uniforms are protected members of IShader (reference include/IShader.hpp:39-45).
template <class S>
struct Uniforms : S {
    using S::cameraPosition;
    using S::material;
    using S::model;
    using S::mvp;
    using S::viewportMat;
    using S::viewProj;
};

// --------------------------------------------------------------------------------
// Shaders this project adds as IShader subclasses (the reference ships neither).
// They follow the structure of PhongShader (reference include/shaders/shaders.hpp:140-247).
struct BlinnPhongShader : public AR::IShader {
    AR::VertexOutput vertex(const AR::Vertex& v, int) override {
        AR::VertexOutput o;
        o.uv = v.uv;
        o.worldPos = glm::vec3(model * glm::vec4(v.position, 1.0f));
        o.normal = glm::normalize(glm::vec3(model * glm::vec4(v.normal, 0.0f)));
        return o;
    }
    bool fragment(glm::vec3& bar, glm::vec4& color, const AR::VSTransformedTriangle& tri) override {
        glm::vec2 uv = bar.x * tri[0].uv + bar.y * tri[1].uv + bar.z * tri[2].uv;
        glm::vec3 albedo = glm::vec3(material->diffuseTexture->sample(uv));
        glm::vec3 n = glm::normalize(bar.x * tri[0].normal + bar.y * tri[1].normal + bar.z * tri[2].normal);
        glm::vec3 fragPos = bar.x * tri[0].worldPos + bar.y * tri[1].worldPos + bar.z * tri[2].worldPos;
        glm::vec3 viewDir = glm::normalize(cameraPosition - fragPos);
        glm::vec3 lightDir = -lightDirection;
        glm::vec3 halfway = glm::normalize(lightDir + viewDir);
        glm::vec3 ambient = 0.1f * lightColor;
        float diff = std::max(glm::dot(n, lightDir), 0.0f);
        glm::vec3 diffuse = diff * lightColor;
        float spec = std::pow(std::max(glm::dot(n, halfway), 0.0f), material->specularExponent * 50.0f);
        glm::vec3 specular = 0.5f * spec * lightColor;
        color = glm::vec4((ambient + diffuse + specular) * albedo, 1.0f);
        return false;
    }
    glm::vec3 lightDirection;
    glm::vec3 lightColor;
};

// Per-vertex colour: RGB travels in Vertex::normal and alpha in Vertex::uv.x (the
// reference Vertex has no colour field, include/mesh.hpp:9-14).
struct GouraudShader : public AR::IShader {
    AR::VertexOutput vertex(const AR::Vertex& v, int) override {
        AR::VertexOutput o;
        o.normal = v.normal;
        o.uv = v.uv;
        return o;
    }
    bool fragment(glm::vec3& bar, glm::vec4& color, const AR::VSTransformedTriangle& tri) override {
        glm::vec3 rgb = bar.x * tri[0].normal + bar.y * tri[1].normal + bar.z * tri[2].normal;
        float a = bar.x * tri[0].uv.x + bar.y * tri[1].uv.x + bar.z * tri[2].uv.x;
        color = glm::vec4(rgb, a);
        return false;
    }
};

glm::mat4 load_mat4(const float* m) {
    glm::mat4 r(0.0f);
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) r[c][k] = m[c * 4 + k];
    return r;
}
void store_mat4(const glm::mat4& m, float* out) {
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) out[c * 4 + k] = m[c][k];
}

std::unique_ptr<AR::Texture> make_texture(const axo_texture& t) {
    if (!t.rgba || t.width <= 0 || t.height <= 0) return nullptr;
    // The only public constructor loads a file; give it none (with stderr muted, since
    // it reports the failure) and then install the pixels directly.
    std::fflush(stderr);
    int saved = dup(2);
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) dup2(devnull, 2);
    auto tex = std::make_unique<AR::Texture>(std::string());
    if (saved >= 0) { dup2(saved, 2); close(saved); }
    if (devnull >= 0) close(devnull);
    size_t bytes = size_t(t.width) * size_t(t.height) * 4;
    auto* data = static_cast<unsigned char*>(std::malloc(bytes));  // released by stbi_image_free (free)
    std::memcpy(data, t.rgba, bytes);
    (*tex).*member(TexData{}) = data;
    (*tex).*member(TexWidth{}) = t.width;
    (*tex).*member(TexHeight{}) = t.height;
    (*tex).*member(TexChannels{}) = 4;
    return tex;
}

std::unique_ptr<AR::Material> make_material(const axo_material& m, const std::string& name) {
    auto mat = std::make_unique<AR::Material>();
    mat->name = name;
    mat->diffuseTexture = make_texture(m.diffuse);
    mat->bumpTexture = make_texture(m.bump);
    mat->metallicTexture = make_texture(m.metallic);
    mat->roughnessTexture = make_texture(m.roughness);
    mat->aoTexture = make_texture(m.ao);
    mat->specularExponent = m.specular_exponent;
    return mat;
}

AR::Vertex vertex_at(const axo_mesh& m, uint32_t i) {
    AR::Vertex v;
    v.position = glm::vec3(m.positions[3 * i], m.positions[3 * i + 1], m.positions[3 * i + 2]);
    v.uv = glm::vec2(m.uvs[2 * i], m.uvs[2 * i + 1]);
    v.normal = glm::vec3(m.normals[3 * i], m.normals[3 * i + 1], m.normals[3 * i + 2]);
    if (m.tangents) v.tangent = glm::vec3(m.tangents[3 * i], m.tangents[3 * i + 1], m.tangents[3 * i + 2]);
    if (m.bitangents) v.bitangent = glm::vec3(m.bitangents[3 * i], m.bitangents[3 * i + 1], m.bitangents[3 * i + 2]);
    return v;
}

AR::ClippedVertex load_cv(const float* f) {
    AR::ClippedVertex cv;
    cv.vertex.position = glm::vec3(f[0], f[1], f[2]);
    cv.vertex.uv = glm::vec2(f[3], f[4]);
    cv.vertex.normal = glm::vec3(f[5], f[6], f[7]);
    cv.vertex.tangent = glm::vec3(f[8], f[9], f[10]);
    cv.vertex.bitangent = glm::vec3(f[11], f[12], f[13]);
    cv.clipPos = glm::vec4(f[14], f[15], f[16], f[17]);
    return cv;
}
void store_cv(const AR::ClippedVertex& cv, float* f) {
    const AR::Vertex& v = cv.vertex;
    const float vals[18] = {v.position.x, v.position.y, v.position.z, v.uv.x, v.uv.y,
                            v.normal.x, v.normal.y, v.normal.z, v.tangent.x, v.tangent.y, v.tangent.z,
                            v.bitangent.x, v.bitangent.y, v.bitangent.z,
                            cv.clipPos.x, cv.clipPos.y, cv.clipPos.z, cv.clipPos.w};
    std::memcpy(f, vals, sizeof(vals));
}

AR::Camera make_camera(const axo_camera& c) {
    AR::Camera cam(glm::vec3(c.position[0], c.position[1], c.position[2]),
                   glm::vec3(c.target[0], c.target[1], c.target[2]), c.fov_degrees, c.aspect);
    cam.setViewport(c.viewport[0], c.viewport[1], c.viewport[2], c.viewport[3]);
    cam.update(0.0f);  // the constructor leaves the view matrix at identity until update()
    return cam;
}

template <class S>
void set_lights(S& s, const axo_shader& sh, bool color) {
    if constexpr (requires { s.lightDirection; })
        s.lightDirection = glm::vec3(sh.light_direction[0], sh.light_direction[1], sh.light_direction[2]);
    if constexpr (requires { s.lightColor; }) {
        if (color) s.lightColor = glm::vec3(sh.light_color[0], sh.light_color[1], sh.light_color[2]);
    }
}

std::unique_ptr<AR::IShader> make_shader(const axo_shader& sh) {
    switch (sh.kind) {
        case AXO_FLAT: { auto s = std::make_unique<AR::FlatShader>(); set_lights(*s, sh, false); return s; }
        case AXO_PHONG: { auto s = std::make_unique<AR::PhongShader>(); set_lights(*s, sh, true); return s; }
        case AXO_PBR: { auto s = std::make_unique<AR::PBRShader>(); set_lights(*s, sh, true); return s; }
        case AXO_BLINN_PHONG: { auto s = std::make_unique<BlinnPhongShader>(); set_lights(*s, sh, true); return s; }
        case AXO_GOURAUD: return std::make_unique<GouraudShader>();
        default: return nullptr;
    }
}

template <class S>
int shade_with(const axo_shader& sh, const axo_material& mat, const float* model, const float* viewProj,
               const float* camPos, const float* verts, const float* bar, float* out) {
    Uniforms<S> s;
    set_lights(s, sh, true);
    auto m = make_material(mat, "m");
    s.model = load_mat4(model);
    s.viewProj = load_mat4(viewProj);
    s.mvp = s.viewProj * s.model;
    s.cameraPosition = glm::vec3(camPos[0], camPos[1], camPos[2]);
    s.material = m.get();
    AR::VSTransformedTriangle tri;
    for (int k = 0; k < 3; ++k) {
        const float* f = verts + 14 * k;
        AR::Vertex v;
        v.position = glm::vec3(f[0], f[1], f[2]);
        v.uv = glm::vec2(f[3], f[4]);
        v.normal = glm::vec3(f[5], f[6], f[7]);
        v.tangent = glm::vec3(f[8], f[9], f[10]);
        v.bitangent = glm::vec3(f[11], f[12], f[13]);
        tri.vertices[k] = s.vertex(v, k);
    }
    glm::vec3 b(bar[0], bar[1], bar[2]);
    glm::vec4 c;
    s.fragment(b, c, tri);
    out[0] = c.r; out[1] = c.g; out[2] = c.b; out[3] = c.a;
    return 0;
}


// TiledPipeline::drawMesh (reference src/tiled_pipeline.cpp:143-322) into a caller-owned
// BGRA8 + f32 framebuffer (read and written in place). Each material group is drawn in
// chunks of at most max_faces_per_draw faces, one single-group drawMesh per chunk: the
// reference's 16 MiB triangle arena has a null upstream (include/tiled_pipeline.hpp:98-104,
// src/tiled_pipeline.cpp:126) and throws std::bad_alloc above roughly 35k triangles per
// draw. Chunked draws in face order give the same image as one draw, because both the
// per-tile early-Z (cpp:569) and the merge (cpp:1150) are strict less-than.
// Returns 0 on success, 1 on bad arguments, 2 on a reference exception.
int draw_with_camera(AR::Camera& cam, const axo_mesh* mesh, const float* model, const axo_shader* shader, int width,
                     int height, int threads, int max_faces_per_draw, uint8_t* bgra, float* depth) {
    AR::Framebuffer fb(width, height, true);
    std::memcpy(fb.getColorData(), bgra, size_t(width) * height * 4);
    std::memcpy(fb.getDepthData(), depth, size_t(width) * height * 4);

    AR::Mesh m;
    auto& verts = m.*member(MeshVertices{});
    auto& faces = m.*member(MeshFaces{});
    auto& mats = m.*member(MeshMaterials{});
    auto& groups = m.*member(MeshGroups{});
    verts.resize(mesh->num_vertices);
    for (uint32_t i = 0; i < mesh->num_vertices; ++i) verts[i] = vertex_at(*mesh, i);
    faces.resize(mesh->num_faces);
    for (uint32_t f = 0; f < mesh->num_faces; ++f)
        faces[f].vertexIndices = {mesh->indices[3 * f], mesh->indices[3 * f + 1], mesh->indices[3 * f + 2]};
    for (uint32_t k = 0; k < mesh->num_materials; ++k) {
        std::string name = "m" + std::to_string(k);
        mats[name] = make_material(mesh->materials[k], name);
    }

    auto sh = make_shader(*shader);
    if (!sh) return 1;
    size_t nthreads = threads > 0 ? size_t(threads) : std::max<size_t>(1, std::thread::hardware_concurrency());
    auto pipe = std::make_unique<AR::TiledPipeline>(nthreads, &cam, &fb);
    pipe->setShader(sh.get());
    glm::mat4 M = load_mat4(model);
    size_t chunk = max_faces_per_draw > 0 ? size_t(max_faces_per_draw) : size_t(16384);
    for (uint32_t g = 0; g < mesh->num_groups; ++g) {
        size_t start = mesh->groups[3 * g], count = mesh->groups[3 * g + 1];
        std::string name = "m" + std::to_string(mesh->groups[3 * g + 2]);
        for (size_t s = 0; s < count; s += chunk) {
            groups.assign(1, AR::MaterialGroup{name, start + s, std::min(chunk, count - s)});
            pipe->drawMesh(M, m);
        }
    }
    std::memcpy(bgra, fb.getColorData(), size_t(width) * height * 4);
    std::memcpy(depth, fb.getDepthData(), size_t(width) * height * 4);
    return 0;
}

}  // namespace

// camera.cpp's handleInput (reference src/camera.cpp:102-130) calls two out-of-line Window
// methods defined in window.cpp (Win32, not compiled here); these read the same members
// the Win32 message handler fills in.
bool AR::Window::isMouseButtonDown(int button) const { return (this->*member(WinButtons()))[button]; }
bool AR::Window::isKeyDown(char key) const { return (this->*member(WinKeys()))[static_cast<unsigned char>(key)]; }

namespace {

// A Window whose input members are set directly: storage for the object without running
// its Win32 constructor (only the input members are ever read).
struct FakeWindow {
    alignas(AR::Window) unsigned char bytes[sizeof(AR::Window)] = {};
    AR::Window& get() { return *reinterpret_cast<AR::Window*>(bytes); }
    void set(float mx, float my, int flags) {
        AR::Window& w = get();
        w.*member(WinMouse()) = glm::vec2(mx, my);
        bool(&b)[3] = w.*member(WinButtons());
        bool(&k)[256] = w.*member(WinKeys());
        for (bool& x : b) x = false;
        for (bool& x : k) x = false;
        b[1] = (flags & 1) != 0;
        k[(unsigned char)'W'] = (flags & 2) != 0;
        k[(unsigned char)'S'] = (flags & 4) != 0;
        k[(unsigned char)'A'] = (flags & 8) != 0;
        k[(unsigned char)'D'] = (flags & 16) != 0;
    }
};

}  // namespace

extern "C" {

// A camera script: Camera(position, target, fov, aspect) + setViewport, then per op
// (6 floats: kind, a0..a3, flags) one of update(a0), handleInput(mouse a0 a1; flags bit 0
// right button, bits 1-4 keys W S A D), setPosition, setTarget, setFov, setAspectRatio,
// setViewport; after each op the view, projection, viewProjection (16 floats each) and the
// position (3): 51 floats per op.
int ref_camera_script(const axo_camera* c, const float* ops, int n, float* out) {
    AR::Camera cam(glm::vec3(c->position[0], c->position[1], c->position[2]),
                   glm::vec3(c->target[0], c->target[1], c->target[2]), c->fov_degrees, c->aspect);
    cam.setViewport(c->viewport[0], c->viewport[1], c->viewport[2], c->viewport[3]);
    FakeWindow win;
    for (int i = 0; i < n; ++i) {
        const float* o = ops + 6 * i;
        switch ((int)o[0]) {
            case 0: cam.update(o[1]); break;
            case 1: win.set(o[1], o[2], (int)o[5]); cam.handleInput(win.get()); break;
            case 2: cam.setPosition(glm::vec3(o[1], o[2], o[3])); break;
            case 3: cam.setTarget(glm::vec3(o[1], o[2], o[3])); break;
            case 4: cam.setFov(o[1]); break;
            case 5: cam.setAspectRatio(o[1]); break;
            case 6: cam.setViewport((int)o[1], (int)o[2], (int)o[3], (int)o[4]); break;
            default: return -1;
        }
        float* r = out + 51 * i;
        store_mat4(cam.getViewMatrix(), r);
        store_mat4(cam.getProjectionMatrix(), r + 16);
        store_mat4(cam.getViewProjectionMatrix(), r + 32);
        const glm::vec3 p = cam.getPosition();
        r[48] = p.x;
        r[49] = p.y;
        r[50] = p.z;
    }
    return 0;
}

// view, projection, viewProjection (column-major, 16 floats each) of a reference Camera.
int ref_camera(const axo_camera* c, float* out48) {
    AR::Camera cam = make_camera(*c);
    store_mat4(cam.getViewMatrix(), out48);
    store_mat4(cam.getProjectionMatrix(), out48 + 16);
    store_mat4(cam.getViewProjectionMatrix(), out48 + 32);
    return 0;
}

// Pipeline::clipTriangle on one input triangle (reference src/pipeline.cpp:176-228).
int ref_clip_triangle(const float* in3, float* out24, int* count) {
    std::array<AR::ClippedVertex, AR::MAX_CLIPPED_VERTS> a{};
    for (int k = 0; k < 3; ++k) a[k] = load_cv(in3 + AXO_CV_FLOATS * k);
    size_t n = 3;
    ClipAccess::clipTriangle(n, a);
    for (size_t k = 0; k < n; ++k) store_cv(a[k], out24 + AXO_CV_FLOATS * k);
    *count = int(n);
    return 0;
}

// Triangle(ClippedVertex...) + static isBackface (reference src/tiled_pipeline.cpp:53-72, 89-119).
int ref_triangle(const float* in3, int width, int height, float* out13, int* backface) {
    std::array<AR::ClippedVertex, 3> v{load_cv(in3), load_cv(in3 + 18), load_cv(in3 + 36)};
    *backface = AR::Triangle::isBackface(v[0], v[1], v[2], width, height) ? 1 : 0;
    AR::Triangle t(v, width, height, nullptr);
    const float vals[13] = {t.screenPos[0].x, t.screenPos[0].y, t.screenPos[1].x, t.screenPos[1].y,
                            t.screenPos[2].x, t.screenPos[2].y, t.ndcZ[0], t.ndcZ[1], t.ndcZ[2],
                            t.minX, t.minY, t.maxX, t.maxY};
    std::memcpy(out13, vals, sizeof(vals));
    return 0;
}

// Texture::sample (reference include/texture.hpp:12-34) at n uv pairs -> n RGBA floats.
int ref_sample(const axo_texture* t, const float* uv, int n, float* out) {
    auto tex = make_texture(*t);
    if (!tex) return 1;
    for (int i = 0; i < n; ++i) {
        glm::vec4 c = tex->sample(glm::vec2(uv[2 * i], uv[2 * i + 1]));
        out[4 * i] = c.r; out[4 * i + 1] = c.g; out[4 * i + 2] = c.b; out[4 * i + 3] = c.a;
    }
    return 0;
}

// vertex() on three Vertex records (14 floats each: pos, uv, normal, tangent, bitangent)
// followed by fragment() at barycentrics bar -> unquantised RGBA.
int ref_shade(const axo_shader* sh, const axo_material* mat, const float* model, const float* viewProj,
              const float* camPos, const float* verts, const float* bar, float* out) {
    switch (sh->kind) {
        case AXO_FLAT: return shade_with<AR::FlatShader>(*sh, *mat, model, viewProj, camPos, verts, bar, out);
        case AXO_PHONG: return shade_with<AR::PhongShader>(*sh, *mat, model, viewProj, camPos, verts, bar, out);
        case AXO_PBR: return shade_with<AR::PBRShader>(*sh, *mat, model, viewProj, camPos, verts, bar, out);
        case AXO_BLINN_PHONG: return shade_with<BlinnPhongShader>(*sh, *mat, model, viewProj, camPos, verts, bar, out);
        case AXO_GOURAUD: return shade_with<GouraudShader>(*sh, *mat, model, viewProj, camPos, verts, bar, out);
        default: return 1;
    }
}

// Camera(position, target, fov, aspect) + update(0), then draw_with_camera.
int ref_render(const axo_mesh* mesh, const float* model, const axo_camera* camera, const axo_shader* shader,
               int width, int height, int threads, int max_faces_per_draw, uint8_t* bgra, float* depth,
               float* matrices_out48) {
    try {
        AR::Camera cam = make_camera(*camera);
        if (matrices_out48) {
            store_mat4(cam.getViewMatrix(), matrices_out48);
            store_mat4(cam.getProjectionMatrix(), matrices_out48 + 16);
            store_mat4(cam.getViewProjectionMatrix(), matrices_out48 + 32);
        }
        return draw_with_camera(cam, mesh, model, shader, width, height, threads, max_faces_per_draw, bgra, depth);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "ref_render: reference threw: %s\n", e.what());
        return 2;
    }
}

// Same draw with an explicit view-projection matrix and eye position installed in the
// Camera (what drawMesh reads from it, src/tiled_pipeline.cpp:148-155).
int ref_draw(const axo_mesh* mesh, const float* model, const float* view_proj, const float* cam_pos,
             const axo_shader* shader, int width, int height, int threads, uint8_t* bgra, float* depth) {
    const int max_faces_per_draw = 16384;
    try {
        AR::Camera cam(glm::vec3(cam_pos[0], cam_pos[1], cam_pos[2]), glm::vec3(0.0f, 0.0f, -1.0f), 60.0f,
                       float(width) / float(height));
        cam.setViewport(0, 0, width, height);
        cam.*member(CamViewProj{}) = load_mat4(view_proj);
        cam.*member(CamPosition{}) = glm::vec3(cam_pos[0], cam_pos[1], cam_pos[2]);
        return draw_with_camera(cam, mesh, model, shader, width, height, threads, max_faces_per_draw, bgra, depth);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "ref_draw: reference threw: %s\n", e.what());
        return 2;
    }
}

// AR::Mesh(path) (src/mesh.cpp:8-27, 300-415, 222-298) on an OBJ file: counts of the
// loaded mesh, then its vertices (14 floats: position, uv, normal, tangent, bitangent),
// faces (3 indices) and material groups (start, count) through ref_obj_fetch.
static std::unique_ptr<AR::Mesh> g_obj_mesh;

int ref_obj_load(const char* path, uint32_t* counts3) {
    try {
        g_obj_mesh = std::make_unique<AR::Mesh>(std::string(path));
    } catch (const std::exception& e) {
        std::fprintf(stderr, "ref_obj_load: reference threw: %s\n", e.what());
        return 2;
    }
    counts3[0] = (uint32_t)g_obj_mesh->getVertices().size();
    counts3[1] = (uint32_t)g_obj_mesh->getFaces().size();
    counts3[2] = (uint32_t)g_obj_mesh->getMaterialGroups().size();
    return 0;
}

int ref_obj_fetch(float* verts14, uint32_t* faces3, uint64_t* groups2) {
    if (!g_obj_mesh) return 1;
    size_t k = 0;
    for (const AR::Vertex& v : g_obj_mesh->getVertices()) {
        const float f[14] = {v.position.x, v.position.y, v.position.z, v.uv.x, v.uv.y, v.normal.x, v.normal.y,
                             v.normal.z, v.tangent.x, v.tangent.y, v.tangent.z, v.bitangent.x, v.bitangent.y,
                             v.bitangent.z};
        std::memcpy(verts14 + 14 * k++, f, sizeof(f));
    }
    k = 0;
    for (const AR::Face& f : g_obj_mesh->getFaces()) {
        for (int j = 0; j < 3; ++j) faces3[3 * k + j] = j < (int)f.vertexIndices.size() ? f.vertexIndices[j] : 0u;
        ++k;
    }
    k = 0;
    for (const AR::MaterialGroup& g : g_obj_mesh->getMaterialGroups()) {
        groups2[2 * k] = g.startIndex;
        groups2[2 * k + 1] = g.faceCount;
        ++k;
    }
    return 0;
}

}  // extern "C"
