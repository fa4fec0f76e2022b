// Batched form: many independent draws (each with its own mesh, camera, shader and
// framebuffer) in one persistent kernel launch. Shared by the host planner (batch.cpp)
// and the kernel (batch.cu).
//
// Layout of one batch in HBM (one allocation, 256-byte aligned sections):
//   BatchDraw[count]      per draw: tensor maps of the framebuffer planes, DrawParams whose
//                         scratch points into this batch, clear request
//   UnitRef[units]        per work unit (vertex units, then face units, then tile units,
//                         then clear units): the draw it belongs to and its index inside it
//   vertex caches         per draw: vscreen[V] float4 + vattr[n*V] float4 (n = VAttr<S>::n)
//                         + shading records (kRecFloat4 float4 per face in draw order)
//   LargeTri[large_cap], large_draw[large_cap], LargeItem[item_cap]: shared by all draws
// Work units: 256 vertices (vertex phase), 256 faces in draw order (geometry phase),
// 8 x tiles_per_warp tiles of 16x16 (key-scan + shade phase); the large-triangle phase
// takes items from the shared list.
#pragma once
#include <stdint.h>

#include "device_types.h"

namespace axr {

// Opaque CUtensorMap (128 bytes, 64-byte aligned), filled by cuTensorMapEncodeTiled.
struct alignas(64) TensorMap128 {
    unsigned char bytes[128];
};

constexpr uint32_t kBatchClearColor = 1u;  // clear the colour plane before the draw
constexpr uint32_t kBatchClearDepth = 2u;  // clear the depth plane before the draw
constexpr uint32_t kBatchTma = 4u;         // the tensor maps are valid (width % 4 == 0)
constexpr uint32_t kBatchClearedApart = 8u; // phased form: the clear kernel writes both planes

constexpr uint32_t kVertUnit = 256;
constexpr uint32_t kFaceUnit = 256;
constexpr uint32_t kUnitWarps = 8;  // warps of a 256-thread CTA
constexpr uint32_t kClearUnit = 1u << 16;  // pixels per unit of the phased form's clear kernel

struct alignas(64) BatchDraw {
    TensorMap128 color_map;  // uint32 [height][width], 16x16 box
    TensorMap128 depth_map;  // float  [height][width], 16x16 box
    DrawParams p;
    uint32_t flags;          // kBatch*
    uint32_t clear_bgra;
    float clear_depth;
    uint32_t pad_[13];
};

constexpr uint32_t kErrBarrier = 4u;  // a grid barrier of the batched kernel timed out

struct UnitRef {
    uint32_t draw;   // index into the launch's draw table
    uint32_t local;  // unit index inside the draw
};

// Device-side phase timing of the batched kernel (enabled with the context's profiling):
// accumulated nanoseconds of the four phases and the launches they cover, plus per-launch
// scratch (start, exit counter, barrier completion times).
struct BatchProfile {
    unsigned long long phase_ns[4];
    unsigned long long launches;
    unsigned long long start;
    unsigned long long exits;
    unsigned long long pad_;
    unsigned long long barrier_ns[3];
    unsigned long long pad2_[5];
};

struct BatchParams {
    const BatchDraw* draws;
    const UnitRef* units;         // vert_units + face_units + tile_units entries
    DevCounters* counters;        // the context's counters (grid barrier in bar_count/bar_gen)
    BatchProfile* prof;           // NULL: no phase timing
    const LargeTri* large;
    const LargeItem* items;
    const uint32_t* large_draw;
    uint32_t count;
    uint32_t vert_units, face_units, tile_units;
    uint32_t clear_units;         // phased form: kClearUnit-pixel spans of the full clears
    uint32_t large_cap, item_cap;
    int32_t collect_stats;
    uint32_t tiles_per_warp;      // tiles a warp takes per tile unit (unit = 8 warps x this)
    BinSet bins;                  // binned form: the launch set's bin counts and clipped records
};

// Launch forms of a batch (chosen per batch by the autotuner):
//   kFormPersistent  one cooperative launch: the four phases behind grid barriers
//   kFormPhased      four launches (one per phase), each over the work units of all draws
//   kFormBinned      three launches over the work units of all draws: vertices, faces
//                    (setup and binning), bins (raster, shading and write-out in shared
//                    memory); tile units are bins of 8 tiles, one CTA each
constexpr int kFormPersistent = 0;
constexpr int kFormPhased = 1;
constexpr int kFormBinned = 2;
constexpr uint32_t kPersistentTilesPerWarp = 8;
constexpr uint32_t kPhasedTilesPerWarp = 4;
constexpr uint32_t kSplitMinDraws = 128;  // phased batches of this many draws run as two launch sets
static_assert(kUnitWarps * kPhasedTilesPerWarp <= 32, "a phased tile unit is described by 32-bit tile masks");

}  // namespace axr
