/* Oracle test infrastructure (tests/, smoke() and bench.py's CPU-baseline leg only).
 *
 * Scene description shared by the two CPU oracles:
 *   - ref_*  : the AxiomR reference sources compiled here (oracle/_ref, x86 only), driven
 *              by oracle/ref_harness.cpp;
 *   - port_* : the C restatement of the same algorithm in oracle/port (builds anywhere).
 * Both export the same functions with these structs so a test can run either one on the
 * same seeded inputs. Nothing in the product links against this header.
 */
#ifndef AXO_H
#define AXO_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* RGBA8 image, row 0 first, as stbi_load(..., STBI_rgb_alpha) returns it
 * (reference include/texture.hpp:12-34 samples it with a y flip). width==0: absent. */
typedef struct axo_texture {
    const uint8_t* rgba;
    int32_t width;
    int32_t height;
} axo_texture;

/* reference include/mesh.hpp:20-34 (the parts the built-in shaders read) */
typedef struct axo_material {
    axo_texture diffuse;
    axo_texture bump;
    axo_texture metallic;
    axo_texture roughness;
    axo_texture ao;
    float specular_exponent;
} axo_material;

/* reference include/mesh.hpp:9-18 (Vertex, as separate arrays), 63-65 (Face), 35-39
 * (MaterialGroup: start face, face count, material index). tangents/bitangents may be
 * NULL (read as zero). */
typedef struct axo_mesh {
    uint32_t num_vertices;
    const float* positions;  /* 3 per vertex */
    const float* uvs;        /* 2 per vertex */
    const float* normals;    /* 3 per vertex */
    const float* tangents;   /* 3 per vertex or NULL */
    const float* bitangents; /* 3 per vertex or NULL */
    uint32_t num_faces;
    const uint32_t* indices; /* 3 per face */
    uint32_t num_groups;
    const uint32_t* groups;  /* (start_face, face_count, material) per group */
    uint32_t num_materials;
    const axo_material* materials;
} axo_mesh;

/* Shader kinds. FLAT/PHONG/PBR are the reference's include/shaders/shaders.hpp;
 * BLINN_PHONG and GOURAUD are this project's extensions (the reference has neither). */
enum { AXO_FLAT = 0, AXO_PHONG = 1, AXO_PBR = 2, AXO_BLINN_PHONG = 3, AXO_GOURAUD = 4 };

typedef struct axo_shader {
    int32_t kind;
    float light_direction[3];
    float light_color[3];
} axo_shader;

/* reference src/camera.cpp:30-56 constructor arguments + setViewport. */
typedef struct axo_camera {
    float position[3];
    float target[3];
    float fov_degrees;
    float aspect;
    int32_t viewport[4]; /* x, y, width, height */
} axo_camera;

/* A parsed OBJ model before Mesh::parseModelFile's de-duplication (src/mesh.cpp:300-415):
 * the "v" / "vt" / "vn" pools and, per face line, its corners as 0-based (v, vt, vn)
 * index triples (vt / vn may be -1 or out of range: absent), corners with an invalid v
 * dropped. A de-duplicated vertex is 14 floats: position[3], uv[2], normal[3],
 * tangent[3], bitangent[3]. */
typedef struct axo_obj {
    uint32_t num_positions;
    const float* positions;
    uint32_t num_uvs;
    const float* uvs;
    uint32_t num_normals;
    const float* normals;
    uint32_t num_corners;
    const int32_t* corners;
    uint32_t num_polygons;
    const uint32_t* polygon_sizes;
} axo_obj;
#define AXO_VERTEX_FLOATS 14

/* ClippedVertex (reference include/pipeline.hpp:13-16) flattened to 18 floats:
 * position[3], uv[2], normal[3], tangent[3], bitangent[3], clipPos[4]. */
#define AXO_CV_FLOATS 18
/* Triangle record (reference include/tiled_pipeline.hpp:14-26) flattened to 13 floats:
 * screenPos[6] (x0,y0,x1,y1,x2,y2), ndcZ[3], minX, minY, maxX, maxY. */
#define AXO_TRI_FLOATS 13

#ifdef __cplusplus
}
#endif
#endif
