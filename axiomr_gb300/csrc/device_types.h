// Data layout in device memory (HBM), shared by the host code and the kernels.
//
// Mesh (SoA, one array per attribute, reference include/mesh.hpp:9-18):
//   pos[V]   float4 (x, y, z, 0)   one 16-byte load per vertex gather
//   nrm[V]   float4                 tan[V], bit[V] float4 (optional, NULL reads as 0)
//   uv[V]    float2
//   idx[3F]  uint32                 Face::vertexIndices, 3 per face
//   groups   DevGroup[G]            MaterialGroup (start face, count, material) + the
//                                   group's first position in draw order
// Texture: RGBA8 texels, row 0 first (as stbi_load returns them), one uint32 per texel.
// Framebuffer: color[W*H] uint32 holding B,G,R,A bytes (row 0 = bottom, reference
//   include/framebuffer.hpp:14-21), depth[W*H] float, key[W*H] uint64 (depth|order
//   visibility keys, all-ones between draws), tile_flag[TX*TY] uint32 (16x16 tile holds a
//   key; set by the rasterisers, cleared by the key scan).
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <vector_types.h>

namespace axr {

constexpr int kTile = 16;            // reference TILE_SIZE (include/tiled_pipeline.hpp:28)
constexpr int kMaxClipVerts = 24;    // reference MAX_CLIPPED_VERTS (include/pipeline.hpp:17)
constexpr uint32_t kMaxOrdinal = (1u << 28) - 1;  // faces per draw: tag = ordinal*16 + clip bits
constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;  // no triangle covers the pixel yet

enum ShaderKind : int32_t { kFlat = 0, kPhong = 1, kPBR = 2, kBlinnPhong = 3, kGouraud = 4 };

// float4s of cached vertex-shader outputs per vertex for a shader kind.
constexpr int vattr_float4s(int shader) {
    return (shader == kPhong || shader == kPBR) ? 4 : (shader == kBlinnPhong ? 2 : 1);
}

struct DevTexture {
    const uint32_t* texels;
    int32_t width, height;
};

struct DevMaterial {
    DevTexture diffuse, bump, metallic, roughness, ao;
    float specular_exponent;
    float pad_[3];
};

struct DevGroup {
    uint32_t start;     // first face index
    uint32_t count;     // faces
    uint32_t base;      // position of the first face in draw order
    uint32_t material;  // index into the material table
};

struct DevMesh {
    const float4* pos;
    const float4* nrm;
    const float4* tan;
    const float4* bit;
    const float2* uv;
    const uint32_t* idx;
    const DevGroup* groups;
    const DevMaterial* materials;
    uint32_t num_vertices, num_faces, num_groups, num_drawn;
};

struct DevTarget {
    uint32_t* color;
    float* depth;
    unsigned long long* key;
    uint32_t* tile_flag;
    int32_t width, height, tiles_x, tiles_y;
};

// Per-draw uniforms (reference include/IShader.hpp:39-45 and the shaders' light fields).
struct DevUniforms {
    float mvp[16];       // viewProj * model, column-major
    float model[16];
    float normal_mat[9]; // mat3(transpose(inverse(model))), FlatShader
    float cam_pos[3];
    float light_dir[3];
    float light_color[3];
    int32_t shader;
    int32_t pad_;
};

// A triangle too large for the per-thread rasteriser: its setup is stored once (64 bytes)
// and each 16x16 tile of its pixel box becomes one work item (LargeItem).
struct LargeTri {
    float e[9];          // edge a, b, c for edges 0..2 after the area-sign flip
    float inv_area;
    float z[3];
    uint32_t tag;        // ordinal * 16 + clip bits: low word of the depth key
    uint16_t x_lo, x_hi, y_lo, y_hi;  // covered pixel range [lo, hi), clipped to the target
};

struct LargeItem {
    uint32_t tri;        // LargeTri index, or kNoItem for a slot reserved but not filled
    uint32_t tile;       // tile index inside the triangle's tile box (row-major)
};
constexpr uint32_t kNoItem = 0xFFFFFFFFu;
constexpr uint32_t kItemsPerGrab = 4;  // tiles a warp takes per atomic

// Bounding box and squared bounding-sphere radius of a mesh's positions, computed on the
// device after an update: lo/hi as order-preserving integers (see kernels.cu), r2 the
// largest squared distance (double) from the box centre.
struct MeshBounds {
    uint32_t lo[3], hi[3];
    unsigned long long r2;  // bits of a non-negative double
};

// Work counters of one draw: the first kCountersReset bytes are zeroed (a memset on
// the stream) before every draw.
struct DevCounters {
    uint32_t large_count;     // LargeTri slots reserved (may exceed the capacity)
    uint32_t item_count;      // LargeItem slots reserved (may exceed the capacity)
    uint32_t item_head;       // next LargeItem to hand out
    uint32_t shade_count;     // covered pixels (unclipped winners) found by the key scan
    uint32_t clip_count;      // covered pixels whose winner is a clipped triangle
    uint32_t bar_count;       // batched kernel: CTAs arrived at the current grid barrier
    uint32_t bar_gen;         // batched kernel: grid barriers completed
    uint32_t error;           // sticky error bits (kErr*), cleared by axr_sync
    unsigned long long stat_triangles;   // triangles that passed clip + cull
    unsigned long long stat_fragments;   // covered (triangle, pixel) pairs
    unsigned long long stat_large;       // triangles sent to the tile rasteriser
    unsigned long long stat_tiles;       // dirty tiles resolved
    unsigned long long stat_tested;      // (triangle, pixel) coverage tests evaluated
    unsigned long long stat_shaded;      // winning fragments shaded
};
static_assert(offsetof(DevCounters, stat_shaded) == offsetof(DevCounters, stat_triangles) + 5 * 8,
              "the six statistics are consecutive (merged as an array)");

constexpr unsigned kCountersReset = 5 * sizeof(uint32_t);
constexpr unsigned kBatchCountersReset = 7 * sizeof(uint32_t);  // + the grid-barrier words
constexpr uint32_t kErrOrdinal = 1u;  // more faces than a depth key can order
constexpr uint32_t kErrIndex = 2u;    // a face indexes a vertex beyond the mesh (face skipped)
constexpr uint32_t kErrTma = 8u;      // a tile load of the binned form did not arrive in time

// Per-vertex cache written by the vertex pass of each draw:
//   vscreen[i] = (screen x, screen y, NDC z, clip-plane masks as uint bits)
//   vattr[n*i ...] = the shader's vertex outputs (n = VAttr<S>::n float4s)
// Resolve work lists written by the key scan: shade[k] = (pixel index, depth-key tag) of a
// covered pixel whose winner is an unclipped triangle; clip_px[k] = the same pair when the
// winner came out of the clipper.
struct DevScratch {
    DevCounters* counters;
    LargeTri* large;
    LargeItem* items;
    float4* vscreen;
    float4* vattr;
    uint2* shade;
    uint2* clip_px;
    uint32_t large_cap;
    uint32_t item_cap;
    uint32_t vcap;
    uint32_t px_cap;          // >= pixels of the target (shade and clip_px capacity)
    int32_t collect_stats;
    int32_t pad_;
    uint32_t* large_draw;     // batched draws: draw index of each LargeTri slot (NULL per draw)
    float4* rec;              // shading records, kRecFloat4 float4 per draw-order position
};

// Shading record of an unclipped triangle that can win a pixel, written by the geometry
// step at its draw-order position and read by the shading step in place of re-deriving the
// setup from the face: the raster record (edge terms, 1/area, vertex depths, pixel range,
// material; x_lo gives the row-start rule of eval_pixel) and the three vertex indices (for
// the cached vertex outputs).
constexpr int kRecFloat4 = 5;

// Binned form: the framebuffer is cut into bins of 8 tiles of 16x16 (tw x th tiles: 8x1,
// 4x2 or 2x4). The face kernel appends each set-up triangle to the entry list of every bin
// its pixel box reaches (less the bins its edges provably miss); the tile kernel then
// rasterises one bin's list into depth keys in shared memory, shades the winners and
// writes the bin's colour and depth once. An entry is a draw-order position (the
// triangle's raster record is rec[position]) or kClipEntry | k for a clipped triangle
// (record k of the launch set's clipped-record list).
constexpr int kBinTiles = 8;
constexpr uint32_t kClipEntry = 0x80000000u;

struct DevBins {
    uint32_t* entries;    // this draw's bins, `cap` entries each (row-major bins)
    uint32_t base;        // index of this draw's bin 0 in the launch set's bin counts
    uint32_t cap;         // entries per bin; a bin offered more spills the rest (see BinSet)
    uint16_t bins_x, bins_y;
    uint8_t tw, th;       // tiles per bin across and down (tw * th == kBinTiles)
    uint16_t thread_px;   // triangle-in-bin rectangles of at most this many pixels are
                          // rasterised by one thread; larger ones by a whole warp
};

// Per launch set (or per context for single draws): zeroed before every launch together
// with the bin counts that follow it in memory.
struct BinCounters {
    uint32_t crec_count;  // clipped-triangle records reserved (may exceed the capacity)
    uint32_t spill;       // (triangle, bin) pairs that found their bin (or the clipped
                          // records) full and went to the framebuffer's key plane instead
    uint32_t pad_[14];
};
static_assert(sizeof(BinCounters) == 64, "bin counts start 64 bytes after the counters");

struct BinSet {
    BinCounters* counters;
    uint32_t* count;      // per bin of the set: entries offered (may exceed the bin's cap)
    float4* crec;         // clipped-triangle raster records, kRasterRec float4 each
    uint32_t nbins;
    uint32_t crec_cap;
};

// Raster record of a set-up triangle (64 bytes): edge a, b, c of edges 0..2 after the
// area-sign flip, 1/area, vertex depths, the covered pixel range [x_lo, x_hi) x [y_lo, y_hi)
// packed as 16-bit pairs, and one word: the material (a shading record at the triangle's
// draw-order position, which adds a fifth float4 with the three vertex indices) or the
// depth-key tag (a clipped triangle's record).
constexpr int kRasterRec = 4;

struct alignas(16) DrawParams {
    DevMesh mesh;
    DevTarget target;
    DevUniforms u;
    DevScratch scratch;
    int32_t small_max_pixels;  // triangles whose pixel box is at most this are rasterised per thread
    uint32_t draw;             // index of the draw in its batch (0 for a single draw)
    DevBins bins;              // binned form only
    uint32_t pad_[2];
};

}  // namespace axr
