// Header-only C++ facade over the C ABI (axr.h) that keeps the AxiomR class names and
// call shapes, so renderer code written against the reference reads the same:
//
//   reference (namespace AR)                 this facade (namespace axr)
//   Framebuffer(w, h, true)                  Framebuffer(ctx, w, h)
//   fb.clearColor(Color) / clearDepth()      same
//   Texture(path)                            Texture(ctx, rgba, w, h)   (decoding is the caller's)
//   Mesh(path)                               Mesh(ctx, MeshData)        (OBJ parsing is the caller's)
//   Camera(pos, target, fov, aspect)         same; update() is implicit
//   FlatShader / PhongShader / PBRShader     same names, lightDirection / lightColor members
//   TiledPipeline(threads, cam, fb)          TiledPipeline(ctx, cam, fb)
//   setShader / setCamera / setFramebuffer   same
//   drawMesh(modelMatrix, mesh)              same (model is 16 floats, column-major)
//   Renderer::drawMesh                       Renderer::drawMesh
//   (no counterpart)                         Draw / Batch: many draws in one launch set
//   (no counterpart)                         Server: the continuous-batching request loop
//
// Failures throw axr::Error (the reference throws std exceptions too); the C ABI itself
// never throws. Every object holds the context it was created on.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "axr.h"

namespace axr {

using Mat4 = std::array<float, 16>;  // column-major
inline Mat4 identity() { return {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}; }

struct Error : std::runtime_error {
    axr_status status;
    Error(axr_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(axr_status s, const axr_context* ctx = nullptr) {
    if (s != AXR_OK) throw Error(s, axr_last_error(ctx));
}

// Color{r, g, b, a} (reference include/math.hpp:17-19)
struct Color {
    unsigned char r, g, b, a;
};

class Context {
public:
    explicit Context(int device = 0) {
        axr_context* c = nullptr;
        check(axr_context_create(device, &c));
        ctx_.reset(c, axr_context_destroy);
    }
    axr_context* get() const { return ctx_.get(); }
    void sync() const { check(axr_sync(ctx_.get()), ctx_.get()); }

private:
    std::shared_ptr<axr_context> ctx_;
};

class Texture {
public:
    Texture(const Context& ctx, const uint8_t* rgba, int width, int height) : ctx_(ctx) {
        axr_texture* t = nullptr;
        check(axr_texture_create(ctx.get(), rgba, width, height, &t), ctx.get());
        tex_.reset(t, [c = ctx_](axr_texture* p) { axr_texture_destroy(c.get(), p); });
    }
    const axr_texture* get() const { return tex_.get(); }

private:
    Context ctx_;
    std::shared_ptr<axr_texture> tex_;
};

// Material (reference include/mesh.hpp:20-34): the textures the shaders read.
struct Material {
    std::shared_ptr<Texture> diffuseTexture, bumpTexture, metallicTexture, roughnessTexture, aoTexture;
    float specularExponent = 1.0f;
};

// MaterialGroup (reference include/mesh.hpp:35-39) with the material by index.
struct MaterialGroup {
    uint32_t startIndex;
    uint32_t faceCount;
    uint32_t material;
};

// Vertex attributes as separate arrays (reference Vertex, include/mesh.hpp:9-18).
struct MeshData {
    std::vector<float> positions, uvs, normals, tangents, bitangents;  // 3, 2, 3, 3, 3 per vertex
    std::vector<uint32_t> indices;                                     // 3 per face
    std::vector<MaterialGroup> groups;                                 // empty: one group, material 0
    std::vector<Material> materials;
};

class Mesh {
public:
    Mesh(const Context& ctx, const MeshData& d) : ctx_(ctx), materials_(d.materials) {
        std::vector<axr_group_desc> groups;
        for (const MaterialGroup& g : d.groups) groups.push_back({g.startIndex, g.faceCount, g.material});
        if (groups.empty()) groups.push_back({0u, uint32_t(d.indices.size() / 3), 0u});
        if (materials_.empty()) materials_.emplace_back();
        std::vector<axr_material_desc> mats;
        auto t = [](const std::shared_ptr<Texture>& p) { return p ? p->get() : nullptr; };
        for (const Material& m : materials_)
            mats.push_back({t(m.diffuseTexture), t(m.bumpTexture), t(m.metallicTexture), t(m.roughnessTexture),
                            t(m.aoTexture), m.specularExponent});
        axr_mesh_desc desc{};
        desc.num_vertices = uint32_t(d.positions.size() / 3);
        desc.positions = d.positions.data();
        desc.uvs = d.uvs.data();
        desc.normals = d.normals.data();
        desc.tangents = d.tangents.empty() ? nullptr : d.tangents.data();
        desc.bitangents = d.bitangents.empty() ? nullptr : d.bitangents.data();
        desc.num_faces = uint32_t(d.indices.size() / 3);
        desc.indices = d.indices.data();
        desc.num_groups = uint32_t(groups.size());
        desc.groups = groups.data();
        desc.num_materials = uint32_t(mats.size());
        desc.materials = mats.data();
        axr_mesh* m = nullptr;
        check(axr_mesh_create(ctx.get(), &desc, &m), ctx.get());
        mesh_.reset(m, [c = ctx_](axr_mesh* p) { axr_mesh_destroy(c.get(), p); });
    }
    const axr_mesh* get() const { return mesh_.get(); }

private:
    Context ctx_;
    std::vector<Material> materials_;  // keeps the textures alive
    std::shared_ptr<axr_mesh> mesh_;
};

class Framebuffer {
public:
    Framebuffer(const Context& ctx, int width, int height) : ctx_(ctx), width_(width), height_(height) {
        axr_framebuffer* f = nullptr;
        check(axr_framebuffer_create(ctx.get(), width, height, &f), ctx.get());
        fb_.reset(f, [c = ctx_](axr_framebuffer* p) { axr_framebuffer_destroy(c.get(), p); });
    }
    void clearColor(const Color& c) { check(axr_framebuffer_clear_color(ctx_.get(), fb_.get(), c.r, c.g, c.b, c.a), ctx_.get()); }
    void clearDepth(float v = std::numeric_limits<float>::infinity()) {
        check(axr_framebuffer_clear_depth(ctx_.get(), fb_.get(), v), ctx_.get());
    }
    // BGRA bytes (width*height*4) and depth (width*height) into host memory; blocks.
    void read(uint8_t* bgra, float* depth) const { check(axr_framebuffer_read(ctx_.get(), fb_.get(), bgra, depth), ctx_.get()); }
    // The colour plane as a PNG file (RGB, top row first: what the reference's window shows;
    // channels 4 = RGBA), encoded on the GPU.
    std::vector<uint8_t> readPng(uint32_t channels = 3) const {
        std::vector<uint8_t> file(axr_png_bound(uint32_t(width_), uint32_t(height_), channels));
        const axr_framebuffer* f = fb_.get();
        void* out = file.data();
        const uint64_t cap = file.size();
        uint64_t size = 0;
        check(axr_framebuffers_read_png(ctx_.get(), 1, &f, channels, &out, &cap, &size), ctx_.get());
        file.resize(size_t(size));
        return file;
    }
    uint32_t getWidth() const { return uint32_t(width_); }
    uint32_t getHeight() const { return uint32_t(height_); }
    axr_framebuffer* get() const { return fb_.get(); }

private:
    Context ctx_;
    int width_, height_;
    std::shared_ptr<axr_framebuffer> fb_;
};

// Camera (reference include/camera.hpp, src/camera.cpp) on the library's camera state: the
// reference's setters, handleInput and update(deltaTime), bit for bit. The constructor
// also runs update(0), as a frame loop does before its first frame (the reference
// constructor leaves the view matrix at identity until an update).
struct InputState {  // what Camera::handleInput reads from the Window
    float mouseX = 0, mouseY = 0;
    bool rightButton = false;
    std::array<bool, 256> keys{};  // indexed by the key's character ('W', 'A', 'S', 'D')
};

class Camera {
public:
    Camera(std::array<float, 3> position = {0, 0, 0}, std::array<float, 3> target = {0, 0, -1}, float fov = 60.0f,
           float aspectRatio = 16.0f / 9.0f) {
        check(axr_camera_init(&s_, position.data(), target.data(), fov, aspectRatio));
        update(0.0f);
    }
    void setPosition(std::array<float, 3> p) { check(axr_camera_set_position(&s_, p.data())); }
    void setTarget(std::array<float, 3> t) { check(axr_camera_set_target(&s_, t.data())); }
    void setFov(float fov) { check(axr_camera_set_fov(&s_, fov)); }
    void setAspectRatio(float a) { check(axr_camera_set_aspect_ratio(&s_, a)); }
    void setViewport(int x, int y, int width, int height) { check(axr_camera_set_viewport(&s_, x, y, width, height)); }
    void handleInput(const InputState& in) {
        axr_input_state st{};
        st.mouse[0] = in.mouseX;
        st.mouse[1] = in.mouseY;
        st.mouse_buttons[1] = in.rightButton ? 1 : 0;
        for (int k = 0; k < 256; ++k) st.keys[k] = in.keys[size_t(k)] ? 1 : 0;
        check(axr_camera_handle_input(&s_, &st));
    }
    void update(float deltaTime) { check(axr_camera_update(&s_, deltaTime)); }
    Mat4 getViewMatrix() const { return to_mat(s_.view); }
    Mat4 getProjectionMatrix() const { return to_mat(s_.projection); }
    Mat4 getViewProjectionMatrix() const { return to_mat(s_.view_proj); }
    Mat4 getViewportMatrix() const { return to_mat(desc().viewport); }
    std::array<float, 3> getPosition() const { return {s_.position[0], s_.position[1], s_.position[2]}; }
    axr_camera_desc desc() const {
        axr_camera_desc d{};
        check(axr_camera_describe(&s_, &d));
        return d;
    }
    const axr_camera_state& state() const { return s_; }

private:
    static Mat4 to_mat(const float* m) {
        Mat4 r{};
        std::copy(m, m + 16, r.begin());
        return r;
    }
    axr_camera_state s_{};
};

// Shaders (reference include/shaders/shaders.hpp) as descriptors.
struct IShader {
    virtual ~IShader() = default;
    virtual axr_shader_desc desc() const = 0;
};
struct FlatShader : IShader {
    std::array<float, 3> lightDirection{0, -1, 0};
    axr_shader_desc desc() const override {
        return {AXR_SHADER_FLAT, {lightDirection[0], lightDirection[1], lightDirection[2]}, {0, 0, 0}};
    }
};
struct LitShader : IShader {
    std::array<float, 3> lightDirection{0, -1, 0};
    std::array<float, 3> lightColor{0.6f, 0.6f, 0.6f};
    virtual int32_t kind() const = 0;
    axr_shader_desc desc() const override {
        return {kind(), {lightDirection[0], lightDirection[1], lightDirection[2]},
                {lightColor[0], lightColor[1], lightColor[2]}};
    }
};
struct PhongShader : LitShader { int32_t kind() const override { return AXR_SHADER_PHONG; } };
struct PBRShader : LitShader { int32_t kind() const override { return AXR_SHADER_PBR; } };
struct BlinnPhongShader : LitShader { int32_t kind() const override { return AXR_SHADER_BLINN_PHONG; } };
struct GouraudShader : IShader {
    axr_shader_desc desc() const override { return {AXR_SHADER_GOURAUD, {0, 0, 0}, {0, 0, 0}}; }
};

// TiledPipeline (reference include/tiled_pipeline.hpp:58-62, include/pipeline.hpp:18-48).
class TiledPipeline {
public:
    TiledPipeline(const Context& ctx, Camera* cam = nullptr, Framebuffer* fb = nullptr) : ctx_(ctx) {
        setCamera(cam);
        setFramebuffer(fb);
    }
    void setShader(const IShader* s) {
        if (!s) {
            check(axr_set_shader(ctx_.get(), nullptr), ctx_.get());
            return;
        }
        axr_shader_desc d = s->desc();
        check(axr_set_shader(ctx_.get(), &d), ctx_.get());
    }
    void setCamera(const Camera* c) {
        if (!c) {
            check(axr_set_camera(ctx_.get(), nullptr), ctx_.get());
            return;
        }
        axr_camera_desc d = c->desc();
        check(axr_set_camera(ctx_.get(), &d), ctx_.get());
    }
    void setFramebuffer(Framebuffer* fb) { check(axr_set_framebuffer(ctx_.get(), fb ? fb->get() : nullptr), ctx_.get()); }
    void drawMesh(const Mat4& modelMatrix, const Mesh& mesh) {
        check(axr_draw_mesh(ctx_.get(), mesh.get(), modelMatrix.data()), ctx_.get());
    }

private:
    Context ctx_;
};

// Renderer::drawMesh (reference src/renderer.cpp:16-19)
class Renderer {
public:
    explicit Renderer(TiledPipeline& p) : pipeline_(p) {}
    void drawMesh(const Mat4& transMat, const Mesh& mesh) { pipeline_.drawMesh(transMat, mesh); }

private:
    TiledPipeline& pipeline_;
};

// ---------------------------------------------------------------- batched form
// One draw of a batch: its own mesh, framebuffer, camera, shader and model matrix; the
// optional clears run before it (fused into the batch's tile pass).
struct Draw {
    const Mesh* mesh = nullptr;
    Framebuffer* framebuffer = nullptr;
    const Camera* camera = nullptr;
    const IShader* shader = nullptr;
    Mat4 model = identity();
    bool clear_color = true, clear_depth = true;
    Color color{0, 0, 0, 255};
    float depth = std::numeric_limits<float>::infinity();

    axr_draw_desc desc() const {
        axr_draw_desc d{};
        d.mesh = mesh->get();
        d.framebuffer = framebuffer->get();
        for (int k = 0; k < 16; ++k) d.model[k] = model[(size_t)k];
        d.camera = camera->desc();
        d.shader = shader->desc();
        d.clear_flags = (clear_color ? AXR_DRAW_CLEAR_COLOR : 0u) | (clear_depth ? AXR_DRAW_CLEAR_DEPTH : 0u);
        d.clear_rgba[0] = color.r;
        d.clear_rgba[1] = color.g;
        d.clear_rgba[2] = color.b;
        d.clear_rgba[3] = color.a;
        d.clear_depth = depth;
        return d;
    }
};

inline std::vector<axr_draw_desc> descs(const std::vector<Draw>& draws) {
    std::vector<axr_draw_desc> d;
    d.reserve(draws.size());
    for (const Draw& x : draws) d.push_back(x.desc());
    return d;
}

// A planned batch: launch() enqueues all its draws (replayable from a CUDA graph).
class Batch {
public:
    Batch(const Context& ctx, const std::vector<Draw>& draws) : ctx_(ctx) {
        std::vector<axr_draw_desc> d = descs(draws);
        axr_batch* b = nullptr;
        check(axr_batch_create(ctx.get(), d.data(), (int32_t)d.size(), &b), ctx.get());
        batch_.reset(b, [c = ctx_](axr_batch* p) { axr_batch_destroy(c.get(), p); });
    }
    void launch() { check(axr_batch_launch(ctx_.get(), batch_.get()), ctx_.get()); }
    axr_batch* get() const { return batch_.get(); }

private:
    Context ctx_;
    std::shared_ptr<axr_batch> batch_;
};

// Tunes the context's launch form and per-density-class raster parameter on `draws`.
inline void autotune(const Context& ctx, const std::vector<Draw>& draws, int repeats = 3) {
    std::vector<axr_draw_desc> d = descs(draws);
    check(axr_batch_autotune(ctx.get(), d.data(), (int32_t)d.size(), repeats, nullptr), ctx.get());
}

// ---------------------------------------------------------------- serving loop
class Server {
public:
    explicit Server(const axr_server_config& cfg) {
        axr_server* s = nullptr;
        check(axr_server_create(&cfg, &s));
        srv_.reset(s, axr_server_destroy);
    }
    int addTexture(const uint8_t* rgba, int width, int height) {
        int32_t id = -1;
        check_(axr_server_add_texture(srv_.get(), rgba, width, height, &id));
        return id;
    }
    int addMesh(const axr_server_mesh_desc& desc) {
        int32_t id = -1;
        check_(axr_server_add_mesh(srv_.get(), &desc, &id));
        return id;
    }
    uint64_t submit(const axr_server_request& req) {
        uint64_t t = 0;
        check_(axr_server_submit(srv_.get(), &req, &t));
        return t;
    }
    axr_server_result wait(uint64_t ticket, int timeout_ms = -1) {
        axr_server_result r{};
        check_(axr_server_wait(srv_.get(), ticket, timeout_ms, &r));
        return r;
    }
    axr_server_stats stats() {
        axr_server_stats s{};
        check_(axr_server_get_stats(srv_.get(), &s));
        return s;
    }
    static uint64_t now() { return axr_server_now_ns(); }

private:
    void check_(axr_status s) {
        if (s != AXR_OK) throw Error(s, axr_server_last_error(srv_.get()));
    }
    std::shared_ptr<axr_server> srv_;
};

}  // namespace axr
