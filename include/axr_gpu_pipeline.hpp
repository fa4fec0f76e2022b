// The reference-side binding: an AR::Pipeline whose drawMesh runs on the GB300 library.
//
// A maintainer adds this header to AxiomR and, in Renderer::init (src/renderer.cpp:71),
// replaces `new TiledPipeline(threads, camera, framebuffer)` with
// `new GpuPipeline(camera, framebuffer)`; nothing else changes. It overrides the virtual
// Pipeline::drawMesh(const glm::mat4&, const Mesh&) (include/pipeline.hpp:25) and reads the
// state the reference's setters hold (m_Shader, m_Camera, m_Framebuffer; pipeline.hpp:27-30).
// It is compiled against the reference's own headers (pipeline.hpp, camera.hpp,
// framebuffer.hpp, mesh.hpp, shaders/shaders.hpp) plus include/axr.h, and links libaxr.so.
//
// Per draw it mirrors TiledPipeline::drawMesh (src/tiled_pipeline.cpp:143-322):
//   * no shader, camera or framebuffer -> nothing happens (tiled_pipeline.cpp:146);
//   * the shader object becomes a kind + uniforms (FlatShader, PhongShader, PBRShader;
//     shaders.hpp:19, 140, 252) with its public lightDirection / lightColor;
//   * the camera's view-projection and viewport matrices and position (camera.hpp:19-23);
//   * the host framebuffer (already cleared by the renderer, src/renderer.cpp:124-125) is
//     written to the device, drawn into and read back, so the renderer's present path
//     (Framebuffer::getColorData) is untouched;
//   * each Mesh is uploaded once, keyed by its address: SoA vertex arrays from
//     Mesh::getVertices, three indices per Face, the MaterialGroups with their materials'
//     textures (rebuilt as RGBA8 from Texture::getPixelRGBA, row 0 first, as stbi_load
//     gives them) and specular exponents.
// Status codes of the C ABI are kept in lastStatus() (the reference's drawMesh returns
// nothing); a GPU that cannot be opened leaves the pipeline inert.
#pragma once

#include <cmath>
#include <cstring>
#include <memory>
#include <unordered_map>
#include <vector>

#include "axr.h"
#include "camera.hpp"
#include "framebuffer.hpp"
#include "mesh.hpp"
#include "pipeline.hpp"
#include "shaders/shaders.hpp"

namespace AR {

class GpuPipeline : public Pipeline {
public:
    GpuPipeline(Camera* cam, Framebuffer* fb, int device = 0) : Pipeline(cam, fb) {
        status_ = axr_context_create(device, &ctx_);
        if (status_ != AXR_OK) ctx_ = nullptr;
    }
    ~GpuPipeline() {
        if (!ctx_) return;
        for (auto& m : meshes_) axr_mesh_destroy(ctx_, m.second.mesh);
        for (auto& t : textures_) axr_texture_destroy(ctx_, t.second);
        if (gpu_fb_) axr_framebuffer_destroy(ctx_, gpu_fb_);
        axr_context_destroy(ctx_);
    }
    GpuPipeline(const GpuPipeline&) = delete;
    GpuPipeline& operator=(const GpuPipeline&) = delete;

    void drawMesh(const glm::mat4& modelMatrix, const Mesh& mesh) override {
        if (!m_Shader || !m_Camera || !m_Framebuffer) return;  // src/tiled_pipeline.cpp:146
        if (!ctx_) return;
        axr_shader_desc sh{};
        if (!describeShader(*m_Shader, sh)) {
            status_ = AXR_E_UNSUPPORTED;
            return;
        }
        axr_camera_desc cam{};
        std::memcpy(cam.view_proj, &m_Camera->getViewProjectionMatrix()[0][0], sizeof(cam.view_proj));
        const glm::mat4 vp = m_Camera->getViewportMatrix();
        std::memcpy(cam.viewport, &vp[0][0], sizeof(cam.viewport));
        const glm::vec3 eye = m_Camera->getPosition();
        cam.position[0] = eye.x;
        cam.position[1] = eye.y;
        cam.position[2] = eye.z;
        axr_mesh* gm = meshHandle(mesh);
        if (!gm || !ensureFramebuffer()) return;
        float model[16];
        std::memcpy(model, &modelMatrix[0][0], sizeof(model));
        const bool ok = check(axr_set_shader(ctx_, &sh)) && check(axr_set_camera(ctx_, &cam)) &&
                        check(axr_set_framebuffer(ctx_, gpu_fb_)) &&
                        check(axr_framebuffer_write(ctx_, gpu_fb_, m_Framebuffer->getColorData(),
                                                    m_Framebuffer->getDepthData())) &&
                        check(axr_draw_mesh(ctx_, gm, model));
        if (ok)
            check(axr_framebuffer_read(ctx_, gpu_fb_, m_Framebuffer->getColorData(), m_Framebuffer->getDepthData()));
    }

    axr_status lastStatus() const { return status_; }
    axr_context* context() const { return ctx_; }

    // The C ABI's view of a Mesh (exposed for tests): SoA arrays, three indices per face,
    // groups with material indices, one material per distinct material name.
    struct MeshArrays {
        std::vector<float> positions, uvs, normals, tangents, bitangents;
        std::vector<uint32_t> indices;
        std::vector<axr_group_desc> groups;
        std::vector<const Material*> materials;
    };
    static MeshArrays meshArrays(const Mesh& mesh) {
        MeshArrays a;
        const auto& vs = mesh.getVertices();
        for (const Vertex& v : vs) {
            a.positions.insert(a.positions.end(), {v.position.x, v.position.y, v.position.z});
            a.uvs.insert(a.uvs.end(), {v.uv.x, v.uv.y});
            a.normals.insert(a.normals.end(), {v.normal.x, v.normal.y, v.normal.z});
            a.tangents.insert(a.tangents.end(), {v.tangent.x, v.tangent.y, v.tangent.z});
            a.bitangents.insert(a.bitangents.end(), {v.bitangent.x, v.bitangent.y, v.bitangent.z});
        }
        for (const Face& f : mesh.getFaces())
            for (int k = 0; k < 3; ++k) a.indices.push_back(k < (int)f.vertexIndices.size() ? f.vertexIndices[k] : 0u);
        std::unordered_map<const Material*, uint32_t> index;
        for (const MaterialGroup& g : mesh.getMaterialGroups()) {
            const Material* m = mesh.getMaterial(g.materialName);
            auto it = index.find(m);
            if (it == index.end()) {
                it = index.emplace(m, (uint32_t)a.materials.size()).first;
                a.materials.push_back(m);
            }
            a.groups.push_back(axr_group_desc{(uint32_t)g.startIndex, (uint32_t)g.faceCount, it->second});
        }
        return a;
    }

    // RGBA8 texels of a reference Texture, row 0 first (the bytes stbi_load returned):
    // getPixelRGBA gives byte / 255 as a float, which rounds back to the byte exactly.
    static std::vector<uint8_t> texels(const Texture& t) {
        std::vector<uint8_t> out((size_t)t.getWidth() * (size_t)t.getHeight() * 4);
        for (int y = 0; y < t.getHeight(); ++y)
            for (int x = 0; x < t.getWidth(); ++x) {
                const glm::vec4 c = t.getPixelRGBA(x, y);
                uint8_t* o = &out[((size_t)y * (size_t)t.getWidth() + (size_t)x) * 4];
                o[0] = (uint8_t)std::lround(c.x * 255.0f);
                o[1] = (uint8_t)std::lround(c.y * 255.0f);
                o[2] = (uint8_t)std::lround(c.z * 255.0f);
                o[3] = (uint8_t)std::lround(c.w * 255.0f);
            }
        return out;
    }

private:
    struct Uploaded {
        axr_mesh* mesh;
        size_t vertices, faces;
    };

    bool check(axr_status s) {
        status_ = s;
        return s == AXR_OK;
    }

    // FlatShader, PhongShader or PBRShader -> kind + lights (IShader::vertex/fragment are
    // private virtuals: the kind is all the library needs).
    static bool describeShader(IShader& s, axr_shader_desc& out) {
        auto copy3 = [](float* dst, const glm::vec3& v) {
            dst[0] = v.x;
            dst[1] = v.y;
            dst[2] = v.z;
        };
        if (auto* f = dynamic_cast<FlatShader*>(&s)) {
            out.kind = AXR_SHADER_FLAT;
            copy3(out.light_direction, f->lightDirection);
            return true;
        }
        if (auto* p = dynamic_cast<PhongShader*>(&s)) {
            out.kind = AXR_SHADER_PHONG;
            copy3(out.light_direction, p->lightDirection);
            copy3(out.light_color, p->lightColor);
            return true;
        }
        if (auto* p = dynamic_cast<PBRShader*>(&s)) {
            out.kind = AXR_SHADER_PBR;
            copy3(out.light_direction, p->lightDirection);
            copy3(out.light_color, p->lightColor);
            return true;
        }
        return false;  // DefaultShader and user shaders have no device counterpart
    }

    bool ensureFramebuffer() {
        const int w = (int)m_Framebuffer->getWidth(), h = (int)m_Framebuffer->getHeight();
        if (gpu_fb_ && fb_w_ == w && fb_h_ == h) return true;
        if (gpu_fb_) axr_framebuffer_destroy(ctx_, gpu_fb_);
        gpu_fb_ = nullptr;
        if (!check(axr_framebuffer_create(ctx_, w, h, &gpu_fb_))) return false;
        fb_w_ = w;
        fb_h_ = h;
        return true;
    }

    axr_texture* textureHandle(const Texture* t) {
        if (!t) return nullptr;
        auto it = textures_.find(t);
        if (it != textures_.end()) return it->second;
        const std::vector<uint8_t> px = texels(*t);
        axr_texture* h = nullptr;
        if (!check(axr_texture_create(ctx_, px.data(), t->getWidth(), t->getHeight(), &h))) return nullptr;
        textures_.emplace(t, h);
        return h;
    }

    axr_mesh* meshHandle(const Mesh& mesh) {
        auto it = meshes_.find(&mesh);
        if (it != meshes_.end() && it->second.vertices == mesh.getVertices().size() &&
            it->second.faces == mesh.getFaces().size())
            return it->second.mesh;
        if (it != meshes_.end()) {
            axr_mesh_destroy(ctx_, it->second.mesh);
            meshes_.erase(it);
        }
        const MeshArrays a = meshArrays(mesh);
        std::vector<axr_material_desc> mats;
        for (const Material* m : a.materials)
            mats.push_back(axr_material_desc{textureHandle(m->diffuseTexture.get()), textureHandle(m->bumpTexture.get()),
                                             textureHandle(m->metallicTexture.get()),
                                             textureHandle(m->roughnessTexture.get()), textureHandle(m->aoTexture.get()),
                                             m->specularExponent});
        axr_mesh_desc d{};
        d.num_vertices = (uint32_t)mesh.getVertices().size();
        d.positions = a.positions.data();
        d.uvs = a.uvs.data();
        d.normals = a.normals.data();
        d.tangents = a.tangents.data();
        d.bitangents = a.bitangents.data();
        d.num_faces = (uint32_t)mesh.getFaces().size();
        d.indices = a.indices.data();
        d.num_groups = (uint32_t)a.groups.size();
        d.groups = a.groups.data();
        d.num_materials = (uint32_t)mats.size();
        d.materials = mats.data();
        axr_mesh* h = nullptr;
        if (!check(axr_mesh_create(ctx_, &d, &h))) return nullptr;
        meshes_.emplace(&mesh, Uploaded{h, mesh.getVertices().size(), mesh.getFaces().size()});
        return h;
    }

    axr_context* ctx_ = nullptr;
    axr_status status_ = AXR_OK;
    axr_framebuffer* gpu_fb_ = nullptr;
    int fb_w_ = 0, fb_h_ = 0;
    std::unordered_map<const Mesh*, Uploaded> meshes_;
    std::unordered_map<const Texture*, axr_texture*> textures_;
};

}  // namespace AR
