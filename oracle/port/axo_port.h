/* Oracle test infrastructure: C restatement of AxiomR's TiledPipeline::drawMesh path
 * (reference src/tiled_pipeline.cpp, src/pipeline.cpp, include/shaders/shaders.hpp,
 * include/texture.hpp, src/camera.cpp). Entry points mirror oracle/ref_harness.cpp one
 * for one (port_* vs ref_*), with the structs of oracle/axo.h. The GPU parity tests
 * check the CUDA path against this port; bench.py times it as the CPU baseline. */
#ifndef AXO_PORT_H
#define AXO_PORT_H
#include "axo.h"
#include "vmath.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ClippedVertex (reference include/pipeline.hpp:13-16) */
typedef struct {
    v3 pos;
    v2 uv;
    v3 nrm, tan, bit;
    v4 clip;
} cvert;

#define MAX_CLIPPED_VERTS 24 /* reference include/pipeline.hpp:17 */
#define TILE_SIZE 16         /* reference include/tiled_pipeline.hpp:28 */
#define BATCH_SIZE 8         /* reference include/tiled_pipeline.hpp:30 */

/* VertexOutput (reference include/IShader.hpp:11-17); tbn columns T, B, N */
typedef struct {
    v3 normal;
    v2 uv;
    v3 world;
    v3 tbn[3];
} vsout;

typedef struct {
    int kind;
    v3 light_dir, light_color;
    m4 model, view_proj, mvp;
    m3 normal_mat; /* mat3(transpose(inverse(model))), FlatShader */
    v3 cam_pos;
} shader_state;

void port_camera_matrices(const axo_camera* c, m4* view, m4* proj, m4* view_proj);
int port_clip(cvert* verts, int count); /* in place, returns the new vertex count */
void port_setup(const cvert* v3in, int width, int height, float out13[13]);
int port_backface(const cvert* a, const cvert* b, const cvert* c, int width, int height);
v4 port_tex_sample(const axo_texture* t, v2 uv);
void shader_init(shader_state* s, const axo_shader* sh, const m4* model, const m4* view_proj, v3 cam_pos);
vsout shader_vertex(const shader_state* s, const cvert* v);
v4 shader_fragment(const shader_state* s, const axo_material* mat, v3 bar, const vsout tri[3]);

int port_camera(const axo_camera* c, float* out48);
int port_clip_triangle(const float* in3, float* out24, int* count);
int port_triangle(const float* in3, int width, int height, float* out13, int* backface);
int port_sample(const axo_texture* t, const float* uv, int n, float* out);
int port_shade(const axo_shader* sh, const axo_material* mat, const float* model, const float* view_proj,
               const float* cam_pos, const float* verts, const float* bar, float* out);
int port_draw(const axo_mesh* mesh, const float* model, const float* view_proj, const float* cam_pos,
              const axo_shader* shader, int width, int height, int threads, uint8_t* bgra, float* depth);
/* Vertex de-duplication, fan triangulation and tangent frames of a parsed OBJ model
 * (ingest.c); verts_out holds num_corners * 14 floats, faces_out num_corners * 3. */
int port_obj_ingest(const axo_obj* in, float* verts_out, uint32_t* nv_out, uint32_t* faces_out, uint32_t* nf_out);
int port_render(const axo_mesh* mesh, const float* model, const axo_camera* camera, const axo_shader* shader,
                int width, int height, int threads, int max_faces_per_draw, uint8_t* bgra, float* depth,
                float* matrices_out48);

#ifdef __cplusplus
}
#endif
#endif
