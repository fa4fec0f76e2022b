// Renders one scene through the C++ facade (include/axr.hpp), the way a renderer written
// against AxiomR's classes would: Framebuffer, Texture, Mesh, Camera, a shader, a
// TiledPipeline and Renderer::drawMesh. Reads the scene from argv[1] and writes the
// framebuffer (BGRA bytes, then float depth) to argv[2]. Used by tests/test_gpu_facade.py.
//
// Scene file (little-endian): u32 W, H; i32 shader; f32 light_dir[3], light_color[3],
// cam_pos[3], cam_target[3], fov, aspect, model[16]; u32 V, F; f32 pos[3V], uv[2V],
// nrm[3V]; u32 idx[3F]; u32 texW, texH; u8 rgba[texW*texH*4]; f32 Ns.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <vector>

#include "axr.hpp"

namespace {
struct Reader {
    std::vector<char> buf;
    size_t at = 0;
    template <class T>
    T get() {
        T v;
        std::memcpy(&v, buf.data() + at, sizeof(T));
        at += sizeof(T);
        return v;
    }
    template <class T>
    std::vector<T> vec(size_t n) {
        std::vector<T> v(n);
        std::memcpy(v.data(), buf.data() + at, n * sizeof(T));
        at += n * sizeof(T);
        return v;
    }
};
}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::cerr << "usage: facade_render scene.bin out.bin\n";
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    Reader r{std::vector<char>(std::istreambuf_iterator<char>(in), {})};
    const uint32_t W = r.get<uint32_t>(), H = r.get<uint32_t>();
    const int32_t kind = r.get<int32_t>();
    auto light_dir = r.vec<float>(3), light_color = r.vec<float>(3);
    auto cam_pos = r.vec<float>(3), cam_target = r.vec<float>(3);
    const float fov = r.get<float>(), aspect = r.get<float>();
    auto model_v = r.vec<float>(16);
    const uint32_t V = r.get<uint32_t>(), F = r.get<uint32_t>();
    axr::MeshData md;
    md.positions = r.vec<float>(3ull * V);
    md.uvs = r.vec<float>(2ull * V);
    md.normals = r.vec<float>(3ull * V);
    md.indices = r.vec<uint32_t>(3ull * F);
    const uint32_t tw = r.get<uint32_t>(), th = r.get<uint32_t>();
    auto rgba = r.vec<uint8_t>(size_t(tw) * th * 4);
    const float ns = r.get<float>();

    try {
        axr::Context ctx(0);
        axr::Framebuffer fb(ctx, int(W), int(H));
        axr::Material mat;
        mat.diffuseTexture = std::make_shared<axr::Texture>(ctx, rgba.data(), int(tw), int(th));
        mat.specularExponent = ns;
        md.materials.push_back(mat);
        axr::Mesh mesh(ctx, md);
        axr::Camera cam({cam_pos[0], cam_pos[1], cam_pos[2]}, {cam_target[0], cam_target[1], cam_target[2]}, fov,
                        aspect);
        cam.setViewport(0, 0, int(W), int(H));
        axr::TiledPipeline pipeline(ctx, &cam, &fb);
        std::unique_ptr<axr::IShader> shader;
        if (kind == AXR_SHADER_FLAT) {
            auto s = std::make_unique<axr::FlatShader>();
            s->lightDirection = {light_dir[0], light_dir[1], light_dir[2]};
            shader = std::move(s);
        } else if (kind == AXR_SHADER_GOURAUD) {
            shader = std::make_unique<axr::GouraudShader>();
        } else {
            std::unique_ptr<axr::LitShader> s;
            if (kind == AXR_SHADER_PHONG) s = std::make_unique<axr::PhongShader>();
            else if (kind == AXR_SHADER_PBR) s = std::make_unique<axr::PBRShader>();
            else s = std::make_unique<axr::BlinnPhongShader>();
            s->lightDirection = {light_dir[0], light_dir[1], light_dir[2]};
            s->lightColor = {light_color[0], light_color[1], light_color[2]};
            shader = std::move(s);
        }
        pipeline.setShader(shader.get());
        axr::Renderer renderer(pipeline);
        fb.clearColor(axr::Color{0, 0, 0, 255});  // src/renderer.cpp:113,124-125
        fb.clearDepth();
        axr::Mat4 model;
        std::copy(model_v.begin(), model_v.end(), model.begin());
        renderer.drawMesh(model, mesh);
        std::vector<uint8_t> bgra(size_t(W) * H * 4);
        std::vector<float> depth(size_t(W) * H);
        fb.read(bgra.data(), depth.data());
        std::ofstream out(argv[2], std::ios::binary);
        out.write(reinterpret_cast<const char*>(bgra.data()), std::streamsize(bgra.size()));
        out.write(reinterpret_cast<const char*>(depth.data()), std::streamsize(depth.size() * 4));
    } catch (const axr::Error& e) {
        std::cerr << "axr error " << e.status << ": " << e.what() << "\n";
        return 1;
    }
    return 0;
}
