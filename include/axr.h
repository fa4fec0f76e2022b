/* AxiomR-GB300 C ABI: the AxiomR software-rasterisation draw path on one GB300 GPU.
 *
 * This header is the drop-in boundary for AxiomR's renderer draw path. Each entry point
 * names the reference interface it replaces (paths relative to the AxiomR tree). The
 * library owns all device memory behind the opaque handles; callers own the handles.
 * No C++ types, exceptions or CUDA types cross this boundary: streams are passed as
 * void* (a cudaStream_t), sizes as fixed-width integers.
 *
 * Threading: one axr_context per host thread (calls on a context are serialised by an
 * internal lock). Work is enqueued on the context's CUDA stream in call order;
 * axr_sync() waits for it. Resources (meshes, textures, framebuffers) may be shared by
 * contexts on the same device, but a framebuffer must not be drawn by two contexts at
 * once.
 *
 * Results are bit-identical to the reference's CPU pipeline for coverage and depth-test
 * winners and depth values, and within 1 LSB per 8-bit colour channel.
 */
#ifndef AXR_H
#define AXR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Raised whenever a struct or signature of this header changes; a program built against
 * this header can compare it with axr_abi_version() of the library it loaded. */
#define AXR_ABI_VERSION 4
int32_t axr_abi_version(void);

/* The reference reports failures with exceptions or silently (src/tiled_pipeline.cpp:146,
 * 126; include/thread_pool.hpp:23-24); across a C ABI they become status codes, with a
 * message available from axr_last_error(). */
typedef enum axr_status {
    AXR_OK = 0,
    AXR_E_INVALID = 1,     /* bad argument or handle */
    AXR_E_OOM = 2,         /* device or host allocation failed */
    AXR_E_BUDGET = 3,      /* device-memory budget of the serving loop exceeded */
    AXR_E_TIMEOUT = 4,     /* a bounded wait gave up */
    AXR_E_CUDA = 5,        /* CUDA runtime error (see axr_last_error) */
    AXR_E_UNSUPPORTED = 6, /* no usable GPU / device capability missing */
    AXR_E_CAPACITY = 7,    /* a preset capacity (faces per draw, captured graph) is too small */
    AXR_E_CANCELLED = 8    /* a serving request was cancelled before it was admitted */
} axr_status;

/* Shader kinds. FLAT, PHONG and PBR are the reference's FlatShader, PhongShader and
 * PBRShader (include/shaders/shaders.hpp:19-62, 140-247, 252-423). BLINN_PHONG and
 * GOURAUD are this library's own (the reference has neither): Blinn-Phong follows
 * PhongShader with the half-vector specular term and no normal map; Gouraud
 * interpolates a per-vertex RGBA colour carried as RGB in the vertex normal and A in
 * uv.x (the reference Vertex has no colour field, include/mesh.hpp:9-14). */
typedef enum axr_shader_kind {
    AXR_SHADER_FLAT = 0,
    AXR_SHADER_PHONG = 1,
    AXR_SHADER_PBR = 2,
    AXR_SHADER_BLINN_PHONG = 3,
    AXR_SHADER_GOURAUD = 4
} axr_shader_kind;

typedef struct axr_context axr_context;
typedef struct axr_texture axr_texture;
typedef struct axr_mesh axr_mesh;
typedef struct axr_framebuffer axr_framebuffer;

/* ------------------------------------------------------------------ context
 * Replaces TiledPipeline(threads, Camera*, Framebuffer*) and its thread pool and arenas
 * (include/tiled_pipeline.hpp:58-62, 98-119; src/tiled_pipeline.cpp:123-139): the
 * context holds the pipeline state, a CUDA stream and the device scratch arena. */
axr_status axr_context_create(int32_t device, axr_context** out);
void axr_context_destroy(axr_context* ctx);
/* Message of the last failed call on this context ("" if none). */
const char* axr_last_error(const axr_context* ctx);
/* The context's cudaStream_t (created non-blocking by axr_context_create). */
void* axr_context_stream(axr_context* ctx);
/* Use a caller-owned cudaStream_t instead (NULL restores the context's own stream). */
axr_status axr_context_set_stream(axr_context* ctx, void* stream);
/* Wait for all work enqueued on the context's stream; reports device-side errors. */
axr_status axr_sync(axr_context* ctx);
/* Diagnostic of the failure path of the batched kernel's grid barrier (no reference
 * counterpart): one CTA waits at a barrier that the other CTA never reaches, the bounded
 * wait gives up after timeout_ms (1..10000), and the call returns what axr_sync reports,
 * AXR_E_TIMEOUT; the context stays usable. No GPU fault is involved. */
axr_status axr_diag_barrier_timeout(axr_context* ctx, uint32_t timeout_ms);
/* Pre-size the scratch arena for draws of up to max_faces faces (needed before a draw
 * is captured into a CUDA graph; draws outside a capture grow it on demand). */
axr_status axr_reserve(axr_context* ctx, uint32_t max_faces);

/* Pinned (page-locked) host memory for asynchronous uploads and read-backs. */
void* axr_host_alloc(size_t bytes);
void axr_host_free(void* p);

/* ------------------------------------------------------------------ textures
 * Replaces Texture (include/texture.hpp:7-64, src/texture.cpp:21-36): RGBA8 texels,
 * row 0 first as stbi_load(..., STBI_rgb_alpha) returns them; sampling is the
 * reference's nearest / clamp-to-edge / y-flipped Texture::sample (texture.hpp:12-34). */
axr_status axr_texture_create(axr_context* ctx, const uint8_t* rgba, int32_t width, int32_t height,
                              axr_texture** out);
/* Replace all texels (same size), asynchronously on the context stream. */
axr_status axr_texture_update(axr_context* ctx, axr_texture* tex, const uint8_t* rgba);
void axr_texture_destroy(axr_context* ctx, axr_texture* tex);

/* ------------------------------------------------------------------ meshes
 * Replaces Mesh / Vertex / Face / MaterialGroup / Material (include/mesh.hpp:9-101).
 * Vertex attributes are separate arrays (structure of arrays) instead of the reference's
 * 56-byte interleaved Vertex; indices are 3 per face. A material group draws faces
 * [start_face, start_face + face_count) with one material; draw order is group order,
 * then face order inside the group (src/tiled_pipeline.cpp:176-259). */
typedef struct axr_material_desc {
    const axr_texture* diffuse;   /* map_Kd */
    const axr_texture* bump;      /* map_Bump / bump / norm (Phong, PBR) */
    const axr_texture* metallic;  /* map_Ks / refl (PBR) */
    const axr_texture* roughness; /* map_Ns (PBR) */
    const axr_texture* ao;        /* map_A0 (PBR) */
    float specular_exponent;      /* Ns (Phong, Blinn-Phong use Ns * 50) */
} axr_material_desc;

typedef struct axr_group_desc {
    uint32_t start_face;
    uint32_t face_count;
    uint32_t material;
} axr_group_desc;

typedef struct axr_mesh_desc {
    uint32_t num_vertices;
    const float* positions;  /* 3 per vertex */
    const float* uvs;        /* 2 per vertex */
    const float* normals;    /* 3 per vertex */
    const float* tangents;   /* 3 per vertex, or NULL (zero) */
    const float* bitangents; /* 3 per vertex, or NULL (zero) */
    uint32_t num_faces;
    const uint32_t* indices; /* 3 per face */
    uint32_t num_groups;
    const axr_group_desc* groups;
    uint32_t num_materials;
    const axr_material_desc* materials;
} axr_mesh_desc;

/* The mesh of an OBJ model parsed on the host, de-duplicated, triangulated and given its
 * tangent frames on the device: Mesh::parseModelFile after its text parsing
 * (src/mesh.cpp:300-415) and Mesh::calculateTangentBitangent (src/mesh.cpp:222-298).
 * Corners are the face lines' corners in file order as 0-based (v, vt, vn) triples, vt /
 * vn -1 (or out of range) when absent or not yet defined at that line, corners with an
 * invalid v dropped (as the reference parser skips them); polygon_sizes gives each face
 * line's corner count (a polygon of n >= 3 corners becomes the fan of n-2 triangles);
 * groups count triangulated faces. The result equals what the reference's Mesh holds
 * (vertices in order of first appearance, bit for bit). */
typedef struct axr_obj_desc {
    uint32_t num_positions;
    const float* positions;  /* "v": 3 per entry */
    uint32_t num_uvs;
    const float* uvs;        /* "vt": 2 per entry */
    uint32_t num_normals;
    const float* normals;    /* "vn": 3 per entry */
    uint32_t num_corners;
    const int32_t* corners;  /* 3 per corner */
    uint32_t num_polygons;
    const uint32_t* polygon_sizes;
    uint32_t num_groups;
    const axr_group_desc* groups;
    uint32_t num_materials;
    const axr_material_desc* materials;
} axr_obj_desc;
axr_status axr_mesh_create_from_obj(axr_context* ctx, const axr_obj_desc* obj, axr_mesh** out);
/* A mesh's vertices back on the host as 14 floats each (position, uv, normal, tangent,
 * bitangent; zeros for absent arrays) and/or its faces as 3 indices each; either may be
 * NULL. Blocks. */
axr_status axr_mesh_read(axr_context* ctx, const axr_mesh* mesh, float* vertices14, uint32_t* indices3);
/* Counts of a mesh (any argument NULL to skip). */
axr_status axr_mesh_counts(const axr_mesh* mesh, uint32_t* vertices, uint32_t* faces, uint32_t* drawn);

/* Upload a mesh (host pointers; the call returns after the data has been copied). */
axr_status axr_mesh_create(axr_context* ctx, const axr_mesh_desc* desc, axr_mesh** out);
/* Re-upload vertex attributes and indices of an existing mesh with the same counts,
 * asynchronously on the context stream (host buffers must stay valid until then;
 * pinned memory from axr_host_alloc makes the copies truly asynchronous). The mesh's
 * bounding sphere, used to plan batches, is recomputed from the new positions (on the
 * device for meshes above 8,192 vertices). Do not update a mesh while another context
 * plans or draws with it. */
axr_status axr_mesh_update(axr_context* ctx, axr_mesh* mesh, const axr_mesh_desc* desc);
void axr_mesh_destroy(axr_context* ctx, axr_mesh* mesh);

/* ------------------------------------------------------------------ framebuffers
 * Replaces Framebuffer (include/framebuffer.hpp:9-69, src/framebuffer.cpp:6-42):
 * colour is 4 bytes per pixel in B, G, R, A order, row 0 at the bottom; depth is one
 * float per pixel (NDC z, smaller is nearer). Created cleared like the reference's
 * constructor: colour 0, depth +inf. */
axr_status axr_framebuffer_create(axr_context* ctx, int32_t width, int32_t height, axr_framebuffer** out);
void axr_framebuffer_destroy(axr_context* ctx, axr_framebuffer* fb);
/* Framebuffer::clearColor(Color{r,g,b,a}) (framebuffer.cpp:26-36) */
axr_status axr_framebuffer_clear_color(axr_context* ctx, axr_framebuffer* fb, uint8_t r, uint8_t g, uint8_t b,
                                       uint8_t a);
/* Framebuffer::clearDepth(value) (framebuffer.cpp:38-42; the reference default is +inf) */
axr_status axr_framebuffer_clear_depth(axr_context* ctx, axr_framebuffer* fb, float depth);
/* Copy colour (W*H*4 bytes) and/or depth (W*H floats) to host memory; either may be
 * NULL. Blocks until the data is on the host. */
axr_status axr_framebuffer_read(axr_context* ctx, const axr_framebuffer* fb, uint8_t* bgra, float* depth);
/* Enqueue the same copies without waiting (use pinned memory and axr_sync). */
axr_status axr_framebuffer_read_async(axr_context* ctx, const axr_framebuffer* fb, uint8_t* bgra, float* depth);
/* The copies of axr_framebuffer_read_async for `count` framebuffers in one call (no
 * reference counterpart): bgra[i] / depth[i] (either array, or any entry, may be NULL)
 * receive framebuffer i. The copies run on several internal streams (several copy engines
 * at once) after the work already enqueued on the context stream; work enqueued later
 * waits for them. Use pinned memory and axr_sync. */
axr_status axr_framebuffers_read_async(axr_context* ctx, int32_t count, const axr_framebuffer* const* fbs,
                                       uint8_t* const* bgra, float* const* depth);
/* A read-back on its own copy streams (no reference counterpart), for pipelines:
 * axr_readback_start enqueues the copies of axr_framebuffers_read_async after the work
 * already on the context stream, but work enqueued later on the context stream does NOT
 * wait for them, so the next frames render while these copy; do not draw into these
 * framebuffers again before axr_readback_wait returns (it waits for the copies). */
typedef struct axr_readback axr_readback;
axr_status axr_readback_create(axr_context* ctx, axr_readback** out);
void axr_readback_destroy(axr_context* ctx, axr_readback* rb);
axr_status axr_readback_start(axr_context* ctx, axr_readback* rb, int32_t count, const axr_framebuffer* const* fbs,
                              uint8_t* const* bgra, float* const* depth);
axr_status axr_readback_wait(axr_context* ctx, axr_readback* rb);
/* A packed read-back: the colour planes of `count` framebuffers gathered on the device and
 * copied as one block into `host` (capacity bytes), image after image: AXR_PACKED_BGRA the
 * planes as stored (4 bytes per pixel, framebuffer row 0 first), AXR_PACKED_RGB 3 bytes per
 * pixel with the top row first: the picture the reference's window shows (Window::present,
 * src/window.cpp:70-84). Image i starts at bytes-per-pixel * (pixels of images 0..i-1).
 * Later work on the context stream does not wait for it; axr_readback_wait does. */
#define AXR_PACKED_BGRA 0
#define AXR_PACKED_RGB 1
axr_status axr_readback_start_packed(axr_context* ctx, axr_readback* rb, int32_t count,
                                     const axr_framebuffer* const* fbs, int32_t format, uint8_t* host,
                                     uint64_t capacity);
/* Upload host colour and/or depth into the framebuffer (either may be NULL). */
axr_status axr_framebuffer_write(axr_context* ctx, axr_framebuffer* fb, const uint8_t* bgra, const float* depth);
axr_status axr_framebuffer_size(const axr_framebuffer* fb, int32_t* width, int32_t* height);
/* Device pointers of the colour (uint32 per pixel) and depth planes, for interop. */
axr_status axr_framebuffer_device_pointers(const axr_framebuffer* fb, void** bgra, void** depth);

/* ------------------------------------------------------------------ output encoding
 * Headless counterpart of Window::present (src/window.cpp:70-84), which copies the BGRA8
 * colour plane into a bottom-up 32-bit DIB (src/windows_bitmap.cpp:15-30) and shows it:
 * each framebuffer's colour plane becomes a PNG file, top row first (framebuffer row
 * height-1 is the file's first scanline), channels 3 = RGB8 (the picture the window
 * shows, alpha dropped) or 4 = RGBA8. Lossless; one deflate stream with the fixed Huffman
 * codes and run/row matches, so flat regions compress and detailed ones stay near 3 or 4
 * bytes per pixel.
 *
 * Worst-case file size of a width x height image (0 for bad arguments). */
uint64_t axr_png_bound(uint32_t width, uint32_t height, uint32_t channels);
/* Encode `count` framebuffers into device buffers out[i] (16-byte aligned, capacity[i] >=
 * axr_png_bound) on the context stream, after the work already enqueued there; sizes is
 * a device array of `count` file sizes, written by the encode. Four kernel launches for
 * the whole list. */
axr_status axr_framebuffers_encode_png(axr_context* ctx, int32_t count, const axr_framebuffer* const* fbs,
                                       uint32_t channels, void* const* out, const uint64_t* capacity,
                                       uint64_t* sizes);
/* Encode into internal device buffers and copy the files to host memory: sizes[i] (host)
 * receives file i's size and files[i] (capacity[i] bytes; pinned memory copies fastest)
 * the file. With files NULL only the sizes are returned. AXR_E_INVALID, with the sizes
 * filled in, when a host buffer is too small. Returns when the files are on the host. */
axr_status axr_framebuffers_read_png(axr_context* ctx, int32_t count, const axr_framebuffer* const* fbs,
                                     uint32_t channels, void* const* files, const uint64_t* capacity,
                                     uint64_t* sizes);
/* The same read-back in steps, for pipelines: a batch keeps its files on the device and has
 * its own copy streams. axr_png_batch_encode enqueues the encode of `count` framebuffers on
 * the context stream (after the work already there, and after this batch's previous files
 * were read) and returns at once; axr_png_batch_sizes waits for that encode and returns the
 * file sizes; axr_png_batch_read copies the files to host buffers (capacity[i] bytes each)
 * and returns when they are there. Render and encode batch k+1 while reading batch k. */
typedef struct axr_png_batch axr_png_batch;
axr_status axr_png_batch_create(axr_context* ctx, axr_png_batch** out);
void axr_png_batch_destroy(axr_context* ctx, axr_png_batch* batch);
axr_status axr_png_batch_encode(axr_context* ctx, axr_png_batch* batch, int32_t count,
                                const axr_framebuffer* const* fbs, uint32_t channels);
axr_status axr_png_batch_sizes(axr_context* ctx, axr_png_batch* batch, uint64_t* sizes);
axr_status axr_png_batch_read(axr_context* ctx, axr_png_batch* batch, void* const* files, const uint64_t* capacity);

/* ------------------------------------------------------------------ pipeline state
 * Pipeline::setShader / setCamera / setFramebuffer (include/pipeline.hpp:22-24). The
 * shader object's uniforms become a plain descriptor: the IShader virtuals
 * (include/IShader.hpp:30-46) cannot cross a C ABI. */
typedef struct axr_shader_desc {
    int32_t kind;              /* axr_shader_kind */
    float light_direction[3];  /* lightDirection (shaders.hpp:60, 244, 402) */
    float light_color[3];      /* lightColor (shaders.hpp:245, 403) */
} axr_shader_desc;

/* What drawMesh reads from the Camera (src/tiled_pipeline.cpp:148-155): the
 * view-projection and viewport matrices (column-major) and the eye position. */
typedef struct axr_camera_desc {
    float view_proj[16];
    float viewport[16];
    float position[3];
} axr_camera_desc;

axr_status axr_set_shader(axr_context* ctx, const axr_shader_desc* shader);
axr_status axr_set_camera(axr_context* ctx, const axr_camera_desc* camera);
axr_status axr_set_framebuffer(axr_context* ctx, axr_framebuffer* fb);

/* TiledPipeline::drawMesh(modelMatrix, mesh) (include/tiled_pipeline.hpp:62,
 * src/tiled_pipeline.cpp:143-322), called by Renderer::drawMesh (src/renderer.cpp:16-19).
 * Enqueued on the context stream. Like the reference, a draw with no shader, camera or
 * framebuffer set does nothing (src/tiled_pipeline.cpp:146). */
axr_status axr_draw_mesh(axr_context* ctx, const axr_mesh* mesh, const float model[16]);

/* Forms of axr_draw_mesh; no counterpart in the reference, both give its frame.
 * KEYED is the default: on one large draw (2M triangles at 1920x1080, 200k at 3840x2160)
 * it measured faster; BINNED was faster on a small one (4k triangles at 512x512).
 * BINNED: the reference's binTrianglesToTiles / processTile /
 * mergeTileResults (src/tiled_pipeline.cpp:368-425, 1125-1181) on the GPU. A face kernel
 * sets up every triangle and appends it to the entry list of each bin of 8 tiles (16x16)
 * that its box reaches; one CTA per bin then rasterises the bin's list into depth keys in
 * shared memory, shades the winners and merges them into the framebuffer, whose tiles it
 * loads and stores with TMA tensor copies. KEYED: the visibility of every covered pixel
 * is decided by a 64-bit atomicMin of (depth, draw order) into the framebuffer's key
 * plane in device memory, then a per-pixel pass shades the winners. */
#define AXR_DRAW_BINNED 0
#define AXR_DRAW_KEYED 1
axr_status axr_set_draw_form(axr_context* ctx, int32_t form);
int32_t axr_get_draw_form(const axr_context* ctx);

/* Bin parameters of the binned forms: for axr_draw_mesh (axr_set_bin_params) and per
 * density class of a batch (axr_batch_set_bin_tuning). No counterpart in the reference,
 * whose tile size and worker batch are compile-time constants (TILE_SIZE, BATCH_SIZE,
 * include/tiled_pipeline.hpp:28-31). A bin offered more entries than its capacity
 * rasterises the rest through the framebuffer's key plane (slower, same result). */
typedef struct axr_bin_params {
    int32_t capacity;       /* entries per bin (16..65536); 0 with axr_set_bin_params: sized
                             * per draw from its faces and framebuffer */
    int32_t tiles_x;        /* bin shape: tiles across (1, 2, 4 or 8); 0 with
                             * axr_set_bin_params: chosen per draw from the framebuffer size */
    int32_t thread_pixels;  /* a triangle's part of a bin of at most this many pixels is
                             * rasterised by one thread, a larger part by a warp (1..2048) */
    int32_t tiles_y;        /* tiles down (1, 2, 4 or 8), tiles_x * tiles_y <= 8; 0: the
                             * most that tiles_x allows (8 / tiles_x) */
} axr_bin_params;
axr_status axr_set_bin_params(axr_context* ctx, const axr_bin_params* params);
axr_status axr_get_bin_params(const axr_context* ctx, axr_bin_params* out);

/* No counterpart in the reference. The same draw as axr_draw_mesh for callers that cannot
 * allocate device memory: a renderer recording its frame into a CUDA graph, a real-time
 * loop that forbids allocator calls after start-up, or a host that owns the device-memory
 * budget. Its scratch lives in one fixed device array inside the library (about 32 MiB,
 * reserved on every GPU that loads the library until exit), so the call allocates nothing.
 * Limits: 65536 vertices, 65536 drawn faces, 1024*1024 framebuffer pixels; larger draws
 * return AXR_E_CAPACITY. The first call on a device looks up the array's address, so make
 * it before any stream capture; the address is kept until exit, so do not use this entry
 * point after a cudaDeviceReset. All calls share the array: calls whose work overlaps on
 * the GPU (other streams or contexts) race. Device error bits and statistics reach
 * axr_sync and axr_stats_read as for axr_draw_mesh; stage profiles leave the call out. */
axr_status axr_draw_mesh_noalloc(axr_context* ctx, const axr_mesh* mesh, const float model[16]);

/* ------------------------------------------------------------------ batched form
 * No reference counterpart: the reference renders one mesh per drawMesh call, each a full
 * pass of its pipeline (src/tiled_pipeline.cpp:143-322; src/renderer.cpp:16-19). A batch
 * is many independent draws, each with its own mesh, camera, shader, model matrix and
 * framebuffer, rendered by one persistent cooperative kernel launch per shader kind present
 * in the batch. Every draw's result is the one axr_draw_mesh gives for it (after the
 * optional clears, which are fused into the draw's tile pass). The framebuffers of a batch
 * must be distinct. */
#define AXR_DRAW_CLEAR_COLOR 1u /* Framebuffer::clearColor before the draw */
#define AXR_DRAW_CLEAR_DEPTH 2u /* Framebuffer::clearDepth before the draw */

typedef struct axr_draw_desc {
    const axr_mesh* mesh;
    axr_framebuffer* framebuffer;
    float model[16];
    axr_camera_desc camera;
    axr_shader_desc shader;
    uint32_t clear_flags;   /* AXR_DRAW_CLEAR_* */
    uint8_t clear_rgba[4];  /* clearColor(Color{r, g, b, a}) */
    float clear_depth;      /* clearDepth(value); the reference default is +inf */
} axr_draw_desc;

typedef struct axr_batch axr_batch;

/* Plan a batch: checks the draws, assigns each draw the raster parameters of its density
 * class from the context's tuning table, uploads the draw table and reserves the batch's
 * device scratch (vertex caches of all draws, shared large-triangle lists). Returns after
 * the upload. Meshes, framebuffers and textures must outlive the batch. */
axr_status axr_batch_create(axr_context* ctx, const axr_draw_desc* draws, int32_t count, axr_batch** out);
/* Enqueue the planned batch on the context stream (per shader kind: a counter reset and
 * the launches of its form). Allocates nothing and reads no host memory, so it can be
 * recorded into a CUDA graph (axr_graph_begin / axr_graph_end) and replayed. */
axr_status axr_batch_launch(axr_context* ctx, axr_batch* batch);
void axr_batch_destroy(axr_context* ctx, axr_batch* batch);

/* Launch forms (the autotuner picks one per batch; batches planned afterwards use it):
 * PERSISTENT: one cooperative launch per shader kind, its four phases (vertices, faces,
 * large-triangle tiles, tile pass) behind grid barriers; PHASED: a clear kernel and four
 * launches per shader kind, one per phase, each over the work units of every draw. A
 * phased batch of 128 or more draws runs each shader kind as two launch sets of
 * alternating draws, the second on a side stream of the context (forked from and joined
 * back into its stream, also inside a graph capture), so that the sets' phases overlap. */
#define AXR_BATCH_PERSISTENT 0
#define AXR_BATCH_PHASED 1
/* BINNED: three launches per shader kind over the work units of every draw: vertices,
 * faces (setup and binning, as axr_draw_mesh's binned form) and bins (raster, shading and
 * write-out of one bin of 8 tiles per CTA, the draw's clears fused into it); bin
 * parameters per density class from axr_batch_set_bin_tuning. Large batches run as two
 * launch sets like PHASED. */
#define AXR_BATCH_BINNED 2
axr_status axr_batch_set_form(axr_context* ctx, int32_t form);
int32_t axr_batch_get_form(const axr_context* ctx);

typedef struct axr_batch_info {
    uint32_t draws;
    uint32_t launches;        /* launch sets per axr_batch_launch: one per shader kind, two for a
                               * phased batch of 128+ draws */
    int32_t form;             /* AXR_BATCH_* the batch was planned for */
    uint32_t pad_;
    uint64_t vertices;        /* vertices of all draws */
    uint64_t faces;           /* faces in draw order of all draws */
    uint64_t pixels;          /* framebuffer pixels of all draws */
    uint64_t tiles;           /* 16x16 tiles of all draws */
    uint64_t device_bytes;    /* device memory held by the batch */
} axr_batch_info;
axr_status axr_batch_get_info(const axr_batch* batch, axr_batch_info* out);

/* One-shot form: plan into a batch kept by the context (re-used while it is large enough)
 * and launch it. Not for graph capture (the draw table is uploaded by this call). */
axr_status axr_draw_batch(axr_context* ctx, const axr_draw_desc* draws, int32_t count);

/* Autotuner. First the launch form, timing the whole batch in both forms. Then, per
 * density class, the largest triangle pixel box rasterised by one thread (larger boxes go
 * to the warp-per-tile rasteriser), timing the sub-batch of the given draws in that class
 * with each candidate `repeats` times. A draw's density class is the estimated mean screen
 * area of its front-facing triangles, from the mesh's bounding sphere projected through
 * its camera: class k covers [2^(2k-1), 2^(2k+1)) pixels (class 0 below 2, the last class
 * 512 and above). The form and the table are the context's; batches planned afterwards
 * use them. out_small_max_pixels (optional) receives the table. */
#define AXR_TUNE_CLASSES 6
axr_status axr_batch_autotune(axr_context* ctx, const axr_draw_desc* draws, int32_t count, int32_t repeats,
                              int32_t out_small_max_pixels[AXR_TUNE_CLASSES]);
axr_status axr_batch_get_tuning(const axr_context* ctx, int32_t small_max_pixels[AXR_TUNE_CLASSES]);
axr_status axr_batch_set_tuning(axr_context* ctx, const int32_t small_max_pixels[AXR_TUNE_CLASSES]);
/* Bin parameters per density class of the binned form (capacity 16..65536, never 0). */
axr_status axr_batch_get_bin_tuning(const axr_context* ctx, axr_bin_params out[AXR_TUNE_CLASSES]);
axr_status axr_batch_set_bin_tuning(axr_context* ctx, const axr_bin_params params[AXR_TUNE_CLASSES]);
/* Density class of one draw (the classification the planner uses). */
int32_t axr_draw_density_class(const axr_draw_desc* draw);

/* ------------------------------------------------------------------ serving loop
 * No reference counterpart (the reference renders frames in its application loop,
 * src/renderer.cpp:98-130). A server owns a context on one device and a host thread that
 * runs a continuous-batching render loop: requests (mesh asset, camera, model, shader,
 * resolution, clears) are admitted as device memory and batch slots free up, each
 * admitted group is rendered as one batch (axr_batch_* machinery) while the previous
 * group's read-backs are in flight, and results (BGRA colour and/or depth) are copied to
 * the request's host buffers. Mesh assets and textures are registered once with host
 * copies; the server keeps them resident on the device and evicts the least recently
 * used ones (not pinned by in-flight requests) when the device-memory budget for resident
 * meshes, textures and framebuffers would be exceeded (the loop's batch scratch and
 * per-draw scratch are its working memory, outside the budget). Framebuffers are pooled
 * per resolution. Latency is measured on the server's clock (axr_server_now_ns). */
typedef struct axr_server axr_server;

typedef struct axr_server_config {
    int32_t device;
    uint64_t memory_budget_bytes; /* device memory for resident meshes, textures, framebuffers */
    int32_t max_batch;            /* requests per batch (continuous-batching cap) */
    int32_t max_inflight;         /* batches on the GPU at once (their read-backs overlap) */
    int32_t per_request;          /* 1: render each request alone with the per-draw path
                                     (clearColor, clearDepth, drawMesh), no batching */
    int32_t overlap_kernels;      /* 1: each in-flight slot renders on its own stream and scratch,
                                     so the kernels of two batches can run side by side; 0: the
                                     slots share one stream (kernels in order, copies overlapped) */
} axr_server_config;

/* A texture asset (RGBA8, row 0 first); *out_id receives its id. */
axr_status axr_server_add_texture(axr_server* srv, const uint8_t* rgba, int32_t width, int32_t height,
                                  int32_t* out_id);
/* A mesh asset: arrays as in axr_mesh_desc, materials naming texture asset ids (-1: none);
 * the server keeps host copies. *out_id receives its id. */
typedef struct axr_server_material {
    int32_t diffuse, bump, metallic, roughness, ao; /* texture asset ids or -1 */
    float specular_exponent;
} axr_server_material;
typedef struct axr_server_mesh_desc {
    uint32_t num_vertices;
    const float* positions;
    const float* uvs;
    const float* normals;
    const float* tangents;   /* or NULL */
    const float* bitangents; /* or NULL */
    uint32_t num_faces;
    const uint32_t* indices;
    uint32_t num_groups;
    const axr_group_desc* groups;
    uint32_t num_materials;
    const axr_server_material* materials;
} axr_server_mesh_desc;
axr_status axr_server_add_mesh(axr_server* srv, const axr_server_mesh_desc* desc, int32_t* out_id);

typedef struct axr_server_request {
    int32_t mesh;             /* mesh asset id */
    int32_t width, height;    /* framebuffer resolution */
    float model[16];
    axr_camera_desc camera;
    axr_shader_desc shader;
    uint32_t clear_flags;     /* AXR_DRAW_CLEAR_* */
    uint8_t clear_rgba[4];
    float clear_depth;
    uint64_t arrival_ns;      /* arrival time on the server clock (0: the submit time) */
    uint8_t* out_bgra;        /* host destination of the colour plane (W*H*4), or NULL */
    float* out_depth;         /* host destination of the depth plane (W*H), or NULL */
    uint32_t png_channels;    /* 3 / 4: also (or instead) return the colour plane as an RGB /
                                 RGBA PNG file (axr_framebuffers_read_png), encoded right after
                                 its batch and copied while the next batch renders; 0: none */
    uint8_t* out_png;         /* host destination of the file */
    uint64_t out_png_capacity;/* its bytes; axr_png_bound(W, H, channels) always suffices */
} axr_server_request;

typedef struct axr_server_result {
    int32_t status;           /* axr_status of the request */
    uint32_t batch_size;      /* requests rendered in the same batch */
    uint64_t arrival_ns;      /* server clock */
    uint64_t launch_ns;       /* its batch was launched */
    uint64_t done_ns;         /* its read-back finished */
    uint64_t batch_id;
    uint64_t png_bytes;       /* size of the PNG file (AXR_E_CAPACITY: it did not fit out_png) */
} axr_server_result;

typedef struct axr_server_stats {
    uint64_t submitted, completed, batches;
    uint64_t uploads;         /* assets made resident (meshes and textures) */
    uint64_t evictions;       /* assets evicted to fit the budget */
    uint64_t framebuffers;    /* framebuffers allocated */
    uint64_t resident_bytes;  /* device memory held now */
    uint64_t peak_bytes;
} axr_server_stats;

axr_status axr_server_create(const axr_server_config* cfg, axr_server** out);
/* Stops the loop after the queued requests are done, then frees everything. */
void axr_server_destroy(axr_server* srv);
uint64_t axr_server_now_ns(void);
/* Queue a request; *ticket identifies it. Host buffers must stay valid until it is done. */
axr_status axr_server_submit(axr_server* srv, const axr_server_request* req, uint64_t* ticket);
/* Wait up to timeout_ms (negative: no limit) for a request; AXR_E_TIMEOUT if not done. */
axr_status axr_server_wait(axr_server* srv, uint64_t ticket, int32_t timeout_ms, axr_server_result* out);
axr_status axr_server_get_stats(axr_server* srv, axr_server_stats* out);
/* Cancel a request that is still queued: it completes at once with AXR_E_CANCELLED (its
 * host buffers are not touched; axr_server_wait returns that status). A request already
 * admitted into a batch runs to completion: AXR_E_INVALID, as for an unknown or finished
 * ticket. */
axr_status axr_server_cancel(axr_server* srv, uint64_t ticket);
/* hold != 0: admit nothing (requests queue up; the batches in flight finish); hold == 0:
 * resume, admitting the queue as batches. For draining a node or grouping a burst. */
axr_status axr_server_hold(axr_server* srv, int32_t hold);
/* Message of the server's last failure ("" if none). */
const char* axr_server_last_error(axr_server* srv);

/* ------------------------------------------------------------------ CUDA graphs
 * Record the draws issued on the context between begin and end into a CUDA graph and
 * replay it. Per-draw scratch must be reserved (axr_reserve) and batches planned
 * (axr_batch_create) beforehand. */
typedef struct axr_graph axr_graph;
axr_status axr_graph_begin(axr_context* ctx);
axr_status axr_graph_end(axr_context* ctx, axr_graph** out);
axr_status axr_graph_launch(axr_context* ctx, axr_graph* graph);
void axr_graph_destroy(axr_graph* graph);

/* ------------------------------------------------------------------ camera helpers
 * Camera (src/camera.cpp:30-100, 191-205): matrices of a camera at `position` looking
 * at `target`, vertical field of view in degrees, aspect ratio, near 0.1, far 100, as
 * Camera(position, target, fov, aspect) followed by update(0). */
axr_status axr_camera_matrices(const float position[3], const float target[3], float fov_degrees, float aspect,
                               float view[16], float projection[16], float view_proj[16]);
axr_status axr_viewport_matrix(int32_t x, int32_t y, int32_t width, int32_t height, float out[16]);

/* The reference Camera as caller-owned state (include/camera.hpp:6-67, src/camera.cpp:
 * 30-205): construction, setters, mouse / keyboard input and update(deltaTime), with the
 * reference's float operation order and behaviour, including: the view matrix stays
 * identity until the first update; setFov / setAspectRatio mark the projection dirty but
 * nothing recomputes it, so they do not change the matrices; update rotates only when both
 * mouse deltas are non-zero; movement is the sum of unit direction vectors per second. */
typedef struct axr_camera_state {
    float position[3];
    float orientation[4];      /* quaternion x, y, z, w */
    float forward[3], right[3], up[3];
    float delta_yaw, delta_pitch;  /* degrees per second from the last input */
    float velocity[3];
    float fov_degrees, aspect_ratio, near_plane, far_plane;
    float movement_speed, mouse_sensitivity;
    float last_mouse[2];
    int32_t viewport[4];       /* x, y, width, height */
    float view[16], projection[16], view_proj[16];
    int32_t view_dirty, projection_dirty;
} axr_camera_state;

/* What Camera::handleInput reads from the Window (include/window.hpp:20-22). */
typedef struct axr_input_state {
    float mouse[2];
    uint8_t mouse_buttons[3];  /* left, right, middle */
    uint8_t keys[256];         /* indexed by the key's character, as Window::isKeyDown */
} axr_input_state;

/* Camera(position, target, fov, aspect) */
axr_status axr_camera_init(axr_camera_state* cam, const float position[3], const float target[3], float fov_degrees,
                           float aspect_ratio);
axr_status axr_camera_set_position(axr_camera_state* cam, const float position[3]);
axr_status axr_camera_set_target(axr_camera_state* cam, const float target[3]);
axr_status axr_camera_set_fov(axr_camera_state* cam, float fov_degrees);
axr_status axr_camera_set_aspect_ratio(axr_camera_state* cam, float aspect_ratio);
axr_status axr_camera_set_viewport(axr_camera_state* cam, int32_t x, int32_t y, int32_t width, int32_t height);
/* Camera::handleInput(window) */
axr_status axr_camera_handle_input(axr_camera_state* cam, const axr_input_state* input);
/* Camera::update(deltaTime) */
axr_status axr_camera_update(axr_camera_state* cam, float delta_time);
/* What drawMesh reads from the camera: view-projection, viewport matrix, position. */
axr_status axr_camera_describe(const axr_camera_state* cam, axr_camera_desc* out);

/* ------------------------------------------------------------------ statistics
 * Counters of the draws issued since the last reset (collection slows the kernels a
 * little and is off by default). */
typedef struct axr_draw_stats {
    uint64_t triangles;  /* triangles that survived clipping and culling */
    uint64_t fragments;  /* covered (triangle, pixel) pairs */
    uint64_t large;      /* triangles rasterised by the tile kernel */
    uint64_t tiles;      /* 16x16 tiles resolved */
    uint64_t tested;     /* (triangle, pixel) coverage tests evaluated */
    uint64_t shaded;     /* winning fragments shaded (covered pixels after the depth test) */
} axr_draw_stats;
axr_status axr_stats_enable(axr_context* ctx, int32_t enable);
axr_status axr_stats_read(axr_context* ctx, axr_draw_stats* out); /* synchronises, then resets */

/* ------------------------------------------------------------------ profiling
 * When enabled, every draw records CUDA events on the context stream between its
 * kernels, and every batched launch records device timestamps at its grid barriers;
 * axr_profile_read synchronises and returns the summed device time of each stage since
 * the last read, and the number of kernels the library launched. */
typedef struct axr_profile {
    uint32_t draws;          /* draws recorded */
    uint32_t pad_;
    double vertex_ms;        /* per-vertex transform and vertex shader */
    double geometry_ms;      /* clip, cull, setup, small-triangle raster */
    double large_ms;         /* large-triangle tile raster */
    double scan_ms;          /* dirty-tile key scan */
    double shade_ms;         /* per-pixel resolve and shading */
    double clipped_ms;       /* resolve of pixels won by clipped triangles */
    uint64_t kernel_launches;/* all kernels launched on this context since creation */
    uint64_t batch_launches; /* batched launches timed (including graph replays) */
    double batch_vertex_ms;  /* batched kernel phases: vertices */
    double batch_face_ms;    /*   faces (clip, cull, setup, small-triangle raster) */
    double batch_large_ms;   /*   large-triangle tiles */
    double batch_tile_ms;    /*   tile pass (key scan, shading, write-out; clears of the persistent form) */
    double batch_clear_ms;   /*   clear kernel of the phased form (fully cleared draws) */
} axr_profile;
axr_status axr_profile_enable(axr_context* ctx, int32_t enable);
axr_status axr_profile_read(axr_context* ctx, axr_profile* out);

/* FP32 issue peak (TFLOP/s) measured on the context's device with independent FMA
 * chains over a fully occupied grid: the denominator of the fragment-ALU roofline. No
 * reference counterpart. */
axr_status axr_measure_fp32_peak(axr_context* ctx, double* tflops);

/* ------------------------------------------------------------------ stage access (tests)
 * Every triangle of a draw that survives clipping and culling, as 14 words each:
 * tag (uint32: draw-order position * 16 + clip bits), screen x0 y0 x1 y1 x2 y2, NDC z0..z2,
 * minX, minY, maxX, maxY; unordered. Mirrors the reference's Triangle records
 * (include/tiled_pipeline.hpp:14-26) produced by the clip stage (src/tiled_pipeline.cpp:185-240).
 * Writes min(count, capacity) records to `out` (host) and the count to *count. */
axr_status axr_debug_triangles(axr_context* ctx, const axr_mesh* mesh, const float model[16],
                               const float view_proj[16], int32_t width, int32_t height, float* out,
                               uint32_t capacity, uint32_t* count);
/* Texture::sample at n uv pairs (host arrays) -> n RGBA floats. */
axr_status axr_debug_sample(axr_context* ctx, const axr_texture* tex, const float* uv, int32_t n, float* out);

#ifdef __cplusplus
}
#endif
#endif /* AXR_H */
