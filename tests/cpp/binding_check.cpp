// Driver of the reference-side binding (include/axr_gpu_pipeline.hpp), compiled against the
// reference's own headers and linked with the reference objects and libaxr.so. Loads an OBJ
// model with the reference Mesh loader, prints what the binding hands to the C ABI (counts,
// groups, materials, texels) and runs one drawMesh through Pipeline's virtual interface.
#include <cstdio>

#include "axr_gpu_pipeline.hpp"

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    AR::Framebuffer fb(64, 48, true);
    fb.clearColor(AR::Color{10, 20, 30, 255});
    fb.clearDepth();
    AR::Camera cam(glm::vec3(0.0f, 0.0f, 3.0f), glm::vec3(0.0f), 60.0f, 64.0f / 48.0f);
    cam.setViewport(0, 0, 64, 48);
    cam.update(0.0f);
    AR::Mesh mesh(argv[1]);
    const auto a = AR::GpuPipeline::meshArrays(mesh);
    std::printf("vertices %zu faces %zu indices %zu groups %zu materials %zu\n", mesh.getVertices().size(),
                mesh.getFaces().size(), a.indices.size(), a.groups.size(), a.materials.size());
    for (const auto& g : a.groups) std::printf("group %u %u %u\n", g.start_face, g.face_count, g.material);
    for (const AR::Material* m : a.materials) {
        std::printf("material Ns %g diffuse %d\n", m->specularExponent, m->diffuseTexture ? 1 : 0);
        if (m->diffuseTexture) {
            const auto px = AR::GpuPipeline::texels(*m->diffuseTexture);
            std::printf("texels %dx%d", m->diffuseTexture->getWidth(), m->diffuseTexture->getHeight());
            for (uint8_t b : px) std::printf(" %u", b);
            std::printf("\n");
        }
    }
    AR::FlatShader shader;
    shader.lightDirection = glm::vec3(0.0f, -1.0f, 0.0f);
    AR::GpuPipeline gpu(&cam, &fb);
    AR::Pipeline& pipe = gpu;  // the renderer holds the base class
    pipe.setShader(&shader);
    pipe.drawMesh(glm::mat4(1.0f), mesh);
    const uint8_t* c = fb.getColorData();
    std::printf("context %d status %d corner %u %u %u %u\n", gpu.context() ? 1 : 0, (int)gpu.lastStatus(), c[0], c[1],
                c[2], c[3]);
    return 0;
}
