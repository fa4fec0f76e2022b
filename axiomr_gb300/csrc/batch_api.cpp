// C ABI of the batched form (include/axr.h, "batched form"): planning a batch of draws into
// one device allocation, launching it, draw density classes and the autotuner.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <unordered_set>
#include <vector>

#include "api_internal.h"
#include "api_types.h"
#include "batch.h"
#include "binned.h"

using namespace axr;
using namespace axr_internal;

static_assert(sizeof(CUtensorMap) == sizeof(TensorMap128), "tensor map size");
static_assert(alignof(TensorMap128) >= 64, "tensor maps are 64-byte aligned");

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// Density class of a draw: estimated mean screen area (pixels) of its front-facing
// triangles. The mesh's bounding sphere goes through the model matrix (radius scaled by the
// largest column norm) and the view-projection; its projected ellipse (semi-axes r * |row
// k of viewProj| / w * size / 2) clamped to the framebuffer, over half the faces.
int density_class(const axr_draw_desc& d) {
    const axr_mesh* m = d.mesh;
    const axr_framebuffer* fb = d.framebuffer;
    if (!m || !fb || m->num_drawn == 0) return 0;
    mesh_sync_bounds(m);
    const float* M = d.model;
    const float* c = m->bound_center;
    double wc[3];
    for (int i = 0; i < 3; ++i) wc[i] = (double)M[i] * c[0] + (double)M[4 + i] * c[1] + (double)M[8 + i] * c[2] + M[12 + i];
    double scale = 0.0;
    for (int col = 0; col < 3; ++col)
        scale = std::max(scale, std::sqrt((double)M[4 * col] * M[4 * col] + (double)M[4 * col + 1] * M[4 * col + 1] +
                                          (double)M[4 * col + 2] * M[4 * col + 2]));
    const double r = (double)m->bound_radius * scale;
    const float* V = d.camera.view_proj;
    auto row = [&](int k) { return (double)V[k] * wc[0] + (double)V[4 + k] * wc[1] + (double)V[8 + k] * wc[2] + V[12 + k]; };
    auto row_norm = [&](int k) {
        return std::sqrt((double)V[k] * V[k] + (double)V[4 + k] * V[4 + k] + (double)V[8 + k] * V[8 + k]);
    };
    const double w = row(3);
    if (!(w > r)) return AXR_TUNE_CLASSES - 1;  // the camera is inside or at the sphere
    const double sx = r * row_norm(0) / w * 0.5 * fb->width;
    const double sy = r * row_norm(1) / w * 0.5 * fb->height;
    const double area = std::min(3.14159265358979 * sx * sy, (double)fb->width * (double)fb->height);
    const double per_tri = area / std::max(1.0, 0.5 * (double)m->num_drawn);
    int k = 0;
    for (double lim = 2.0; k < AXR_TUNE_CLASSES - 1 && per_tri >= lim; lim *= 4.0) ++k;
    return k;
}

axr_status check_draws(axr_context* ctx, const axr_draw_desc* draws, int32_t count) {
    if (count < 0 || (count > 0 && !draws)) return fail(ctx, AXR_E_INVALID, "bad draw list");
    std::unordered_set<const axr_framebuffer*> seen;
    seen.reserve((size_t)count * 2);
    for (int32_t i = 0; i < count; ++i) {
        const axr_draw_desc& d = draws[i];
        if (!d.mesh || !d.framebuffer) return fail(ctx, AXR_E_INVALID, "draw %d has no mesh or framebuffer", i);
        if (d.shader.kind < AXR_SHADER_FLAT || d.shader.kind > AXR_SHADER_GOURAUD)
            return fail(ctx, AXR_E_INVALID, "draw %d: unknown shader kind %d", i, d.shader.kind);
        if (d.mesh->device != ctx->device || d.framebuffer->device != ctx->device)
            return fail(ctx, AXR_E_INVALID, "draw %d uses resources of another device", i);
        if (!seen.insert(d.framebuffer).second)
            return fail(ctx, AXR_E_INVALID, "draw %d: the framebuffers of a batch must be distinct", i);
    }
    return AXR_OK;
}

uint32_t ceil_div(uint64_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

// Bins of one draw of a binned batch.
struct BinPlanD {
    uint16_t bins_x = 0, bins_y = 0;
    uint8_t tw = 8, th = 1;
    uint32_t cap = 0;
    uint16_t thread_px = 64;
};

// Build the batch's draw table and launch descriptions into `b`, (re)allocating its device
// memory when it is too small. `async`: upload with cudaMemcpyAsync on the context stream
// (the host table is copied before the call returns); otherwise synchronously.
axr_status plan_batch(axr_context* ctx, const axr_draw_desc* draws, int32_t count, axr_batch* b, bool async) {
    axr_status st = check_draws(ctx, draws, count);
    if (st != AXR_OK) return st;
    // draws grouped by shader kind (one launch each), batch order inside a group
    std::vector<int32_t> order((size_t)count);
    for (int32_t i = 0; i < count; ++i) order[(size_t)i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t x, int32_t y) { return draws[x].shader.kind < draws[y].shader.kind; });
    std::vector<std::pair<int, std::pair<size_t, size_t>>> groups;  // kind, [first, last)
    for (size_t i = 0; i < order.size(); ++i) {
        const int kind = draws[order[i]].shader.kind;
        if (groups.empty() || groups.back().first != kind) groups.push_back({kind, {i, i}});
        groups.back().second.second = i + 1;
    }
    // sizes
    uint64_t faces = 0, verts = 0, pixels = 0, tiles = 0;
    size_t cache_bytes = 0;
    for (int32_t i = 0; i < count; ++i) {
        const axr_draw_desc& d = draws[i];
        faces += d.mesh->num_drawn;
        verts += d.mesh->num_vertices;
        pixels += (uint64_t)d.framebuffer->width * d.framebuffer->height;
        tiles += (uint64_t)d.framebuffer->tiles_x * d.framebuffer->tiles_y;
        const size_t V = d.mesh->num_vertices;
        cache_bytes += align256(16 * V) + align256(16 * V * (size_t)vattr_float4s(d.shader.kind)) +
                       align256(16 * (size_t)kRecFloat4 * d.mesh->num_drawn);
    }
    // shared large-triangle lists: a triangle that finds them full is rasterised by its own
    // thread instead, so the sizes trade memory for speed only
    const uint32_t large_cap_all = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(faces, 65536), 1u << 22);
    const uint32_t item_cap_all = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(4 * faces, 1u << 20), 1u << 24);
    // The phased form of a large batch runs as two launch sets of alternating draws, one on
    // the context stream and one on a side stream, each with its own counters and
    // large-triangle lists (the lists' capacity is shared out): one set's phases fill the
    // other's tails and gaps, e.g. the issue-bound large-triangle phase beside the
    // latency-bound tile pass.
    const bool binned = ctx->batch_form == kFormBinned;
    const int nsets =
        ((ctx->batch_form == kFormPhased || binned) && count >= (int32_t)kSplitMinDraws) ? 2 : 1;
    // binned form: each draw's bin shape and capacity from its density class; per launch set
    // the bins (counts) and bin entries of its draws, and its clipped-triangle records
    std::vector<BinPlanD> bplan((size_t)count);
    uint64_t set_bins[2] = {0, 0}, set_entries[2] = {0, 0}, set_faces[2] = {0, 0};
    if (binned) {
        for (const auto& g : groups)
            for (size_t k = 0; k < g.second.second - g.second.first; ++k) {
                const int set = (int)(k % (size_t)nsets);
                const int32_t i = order[g.second.first + k];
                BinPlanD& bp = bplan[(size_t)i];
                const axr_bin_params& tp = ctx->tune_bin[density_class(draws[i])];
                bin_shape(tp, &bp.tw, &bp.th);
                bin_geometry(draws[i].framebuffer->tiles_x, draws[i].framebuffer->tiles_y, bp.tw, bp.th, &bp.bins_x,
                             &bp.bins_y);
                bp.cap = (uint32_t)tp.capacity;
                bp.thread_px = (uint16_t)tp.thread_pixels;
                set_bins[set] += (uint64_t)bp.bins_x * bp.bins_y;
                set_entries[set] += (uint64_t)bp.bins_x * bp.bins_y * bp.cap;
                set_faces[set] += draws[i].mesh->num_drawn;
            }
    }
    uint32_t set_crec[2];
    for (int s = 0; s < 2; ++s) set_crec[s] = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(1u << 16, set_faces[s] / 4), 1u << 24);
    const uint32_t large_cap = std::max<uint32_t>(65536, (large_cap_all + nsets - 1) / nsets);
    const uint32_t item_cap = std::max<uint32_t>(1u << 20, (item_cap_all + nsets - 1) / nsets);
    // work units of every draw (the same counts as the loop below assigns)
    const int form = ctx->batch_form;
    const uint32_t tiles_per_warp = form == kFormPersistent ? kPersistentTilesPerWarp : kPhasedTilesPerWarp;
    const uint32_t tile_unit = kUnitWarps * tiles_per_warp;
    size_t total_units = 0;
    for (int32_t i = 0; i < count; ++i) {
        const axr_draw_desc& d = draws[i];
        const bool drawn = d.mesh->num_drawn > 0;
        total_units += (drawn ? ceil_div(d.mesh->num_vertices, kVertUnit) : 0u) + ceil_div(d.mesh->num_drawn, kFaceUnit);
        if (binned)
            total_units += (uint64_t)bplan[(size_t)i].bins_x * bplan[(size_t)i].bins_y;
        else if (drawn || (d.clear_flags & (AXR_DRAW_CLEAR_COLOR | AXR_DRAW_CLEAR_DEPTH)))
            total_units += ceil_div((uint64_t)d.framebuffer->tiles_x * d.framebuffer->tiles_y, tile_unit);
        if (form == kFormPhased && (d.clear_flags & AXR_DRAW_CLEAR_COLOR) && (d.clear_flags & AXR_DRAW_CLEAR_DEPTH) &&
            !d.framebuffer->tma)
            total_units += ceil_div((uint64_t)d.framebuffer->width * d.framebuffer->height, kClearUnit);
    }
    const size_t table_bytes = align256(sizeof(BatchDraw) * (size_t)std::max(count, 1));
    const size_t units_bytes = align256(sizeof(UnitRef) * std::max<size_t>(total_units, 1));
    size_t set_list_bytes = align256(sizeof(LargeTri) * (size_t)large_cap) +
                            align256(sizeof(uint32_t) * (size_t)large_cap) +
                            align256(sizeof(LargeItem) * (size_t)item_cap);
    size_t set_bytes[2] = {0, 0};  // binned: counters + counts, entries, clipped records
    if (binned) {
        set_list_bytes = 0;
        for (int s = 0; s < nsets; ++s)
            set_bytes[s] = align256(sizeof(BinCounters) + sizeof(uint32_t) * set_bins[s]) +
                           align256(sizeof(uint32_t) * set_entries[s]) + align256(16 * (size_t)kRasterRec * set_crec[s]);
    }
    const size_t counter_bytes = align256(sizeof(DevCounters));
    const size_t need = table_bytes + units_bytes + align256(cache_bytes) + set_list_bytes * nsets +
                        counter_bytes * (nsets - 1) + set_bytes[0] + set_bytes[1];
    if (need > b->bytes) {
        if (ctx->capturing) return fail(ctx, AXR_E_CAPACITY, "a batch cannot be planned during graph capture");
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        free_batch(b);
        AXR_CUDA(ctx, cudaMalloc(&b->dev, need));
        b->bytes = need;
    }
    unsigned char* base = static_cast<unsigned char*>(b->dev);
    BatchDraw* d_table = reinterpret_cast<BatchDraw*>(base);
    UnitRef* d_units = reinterpret_cast<UnitRef*>(base + table_bytes);
    unsigned char* cache = base + table_bytes + units_bytes;
    unsigned char* lists = cache + align256(cache_bytes);
    LargeTri* d_large[2];
    uint32_t* d_large_draw[2];
    LargeItem* d_items[2];
    DevCounters* d_counters[2] = {ctx->counters, nullptr};
    for (int s = 0; s < nsets; ++s) {
        unsigned char* l = lists + set_list_bytes * (size_t)s;
        d_large[s] = reinterpret_cast<LargeTri*>(l);
        d_large_draw[s] = reinterpret_cast<uint32_t*>(l + align256(sizeof(LargeTri) * (size_t)large_cap));
        d_items[s] = reinterpret_cast<LargeItem*>(reinterpret_cast<unsigned char*>(d_large_draw[s]) +
                                                  align256(sizeof(uint32_t) * (size_t)large_cap));
    }
    if (nsets > 1) {
        d_counters[1] = reinterpret_cast<DevCounters*>(lists + set_list_bytes * (size_t)nsets);
        // statistics and error bits start at zero; the merge after each launch zeroes them again
        AXR_CUDA(ctx, cudaMemsetAsync(d_counters[1], 0, sizeof(DevCounters), ctx->stream));
    }
    BinCounters* d_bin_counters[2] = {nullptr, nullptr};
    uint32_t* d_bin_entries[2] = {nullptr, nullptr};
    float4* d_crec[2] = {nullptr, nullptr};
    if (binned) {
        unsigned char* q = lists + set_list_bytes * (size_t)nsets + counter_bytes * (size_t)(nsets - 1);
        for (int s = 0; s < nsets; ++s) {
            d_bin_counters[s] = reinterpret_cast<BinCounters*>(q);
            q += align256(sizeof(BinCounters) + sizeof(uint32_t) * set_bins[s]);
            d_bin_entries[s] = reinterpret_cast<uint32_t*>(q);
            q += align256(sizeof(uint32_t) * set_entries[s]);
            d_crec[s] = reinterpret_cast<float4*>(q);
            q += align256(16 * (size_t)kRasterRec * set_crec[s]);
        }
    }
    uint64_t set_bin_at[2] = {0, 0}, set_entry_at[2] = {0, 0};  // binned: next bin / entry of each set

    std::vector<BatchDraw> table((size_t)std::max(count, 1));
    std::vector<UnitRef> units;
    units.reserve(total_units);
    b->launches.clear();
    for (const auto& g : groups) {
        const size_t first = g.second.first, last = g.second.second, n = last - first;
        std::vector<UnitRef> set_uv[2], set_uf[2], set_ut[2], set_uc[2];
        const uint64_t group_bin_at[2] = {set_bin_at[0], set_bin_at[1]};  // the launches' first bins
        for (size_t k = 0; k < n; ++k) {
            const int set = (int)(k % (size_t)nsets);
            std::vector<UnitRef>&uv = set_uv[set], &uf = set_uf[set], &ut = set_ut[set], &uc = set_uc[set];
            const axr_draw_desc& d = draws[order[first + k]];
            const axr_mesh* m = d.mesh;
            const axr_framebuffer* fb = d.framebuffer;
            BatchDraw& bd = table[first + k];
            std::memset(&bd, 0, sizeof(bd));
            bd.color_map = fb->color_map;
            bd.depth_map = fb->depth_map;
            DrawParams& p = bd.p;
            p.mesh = DevMesh{m->pos, m->nrm, m->tan, m->bit, m->uv, m->idx, m->groups, m->materials,
                             m->num_vertices, m->num_faces, m->num_groups, m->num_drawn};
            p.target = DevTarget{fb->color, fb->depth, fb->key, fb->tile_flag,
                                 fb->width, fb->height, fb->tiles_x, fb->tiles_y};
            p.u = make_uniforms(d.camera, d.shader, d.model);
            float4* vscreen = reinterpret_cast<float4*>(cache);
            cache += align256(16 * (size_t)m->num_vertices);
            float4* vattr = reinterpret_cast<float4*>(cache);
            cache += align256(16 * (size_t)m->num_vertices * (size_t)vattr_float4s(d.shader.kind));
            float4* rec = reinterpret_cast<float4*>(cache);
            cache += align256(16 * (size_t)kRecFloat4 * m->num_drawn);
            p.scratch = binned ? DevScratch{d_counters[set], nullptr, nullptr, vscreen, vattr, nullptr, nullptr, 0u, 0u,
                                            m->num_vertices, 0u, 0, 0, nullptr, rec}
                               : DevScratch{d_counters[set], d_large[set], d_items[set], vscreen, vattr, nullptr, nullptr,
                                            large_cap, item_cap, m->num_vertices, 0u, 0, 0, d_large_draw[set], rec};
            p.small_max_pixels = ctx->tune_small[density_class(d)];
            p.draw = (uint32_t)k;
            if (binned) {
                const BinPlanD& bp = bplan[(size_t)order[first + k]];
                const uint32_t nb = (uint32_t)bp.bins_x * bp.bins_y;
                p.bins = DevBins{d_bin_entries[set] + set_entry_at[set], (uint32_t)(set_bin_at[set] - group_bin_at[set]),
                                 bp.cap, bp.bins_x, bp.bins_y, bp.tw, bp.th, bp.thread_px};
                set_bin_at[set] += nb;
                set_entry_at[set] += (uint64_t)nb * bp.cap;
            }
            bd.flags = (d.clear_flags & AXR_DRAW_CLEAR_COLOR ? kBatchClearColor : 0u) |
                       (d.clear_flags & AXR_DRAW_CLEAR_DEPTH ? kBatchClearDepth : 0u) | (fb->tma ? kBatchTma : 0u);
            // bytes B, G, R, A (src/framebuffer.cpp:26-36)
            bd.clear_bgra = ((uint32_t)d.clear_rgba[3] << 24) | ((uint32_t)d.clear_rgba[0] << 16) |
                            ((uint32_t)d.clear_rgba[1] << 8) | (uint32_t)d.clear_rgba[2];
            bd.clear_depth = d.clear_depth;
            const bool drawn = m->num_drawn > 0;
            const uint32_t nv = drawn ? ceil_div(m->num_vertices, kVertUnit) : 0u;
            const uint32_t nf = ceil_div(m->num_drawn, kFaceUnit);
            const uint32_t nt = binned ? (uint32_t)p.bins.bins_x * p.bins.bins_y
                                : (drawn || bd.flags & (kBatchClearColor | kBatchClearDepth))
                                    ? ceil_div((uint64_t)fb->tiles_x * fb->tiles_y, tile_unit)
                                    : 0u;
            for (uint32_t j = 0; j < nv; ++j) uv.push_back(UnitRef{(uint32_t)k, j});
            for (uint32_t j = 0; j < nf; ++j) uf.push_back(UnitRef{(uint32_t)k, j});
            for (uint32_t j = 0; j < nt; ++j) ut.push_back(UnitRef{(uint32_t)k, j});
            // the phased form clears both planes of a fully cleared draw in its tile pass:
            // the key-less tiles with TMA stores of a cleared tile. A framebuffer without
            // tensor maps (width not a multiple of 4) is cleared by its own kernel first.
            if (form == kFormPhased && (bd.flags & kBatchClearColor) && (bd.flags & kBatchClearDepth) && !fb->tma) {
                bd.flags |= kBatchClearedApart;
                const uint32_t nc = ceil_div((uint64_t)fb->width * fb->height, kClearUnit);
                for (uint32_t j = 0; j < nc; ++j) uc.push_back(UnitRef{(uint32_t)k, j});
            }
        }
        for (int set = 0; set < nsets; ++set) {
            const std::vector<UnitRef>&uv = set_uv[set], &uf = set_uf[set], &ut = set_ut[set], &uc = set_uc[set];
            const size_t unit_at = units.size();
            units.insert(units.end(), uv.begin(), uv.end());
            units.insert(units.end(), uf.begin(), uf.end());
            units.insert(units.end(), ut.begin(), ut.end());
            units.insert(units.end(), uc.begin(), uc.end());
            axr_batch::Launch L{};
            L.shader = g.first;
            L.set = set;
            BatchParams& bp = L.params;
            bp.draws = d_table + first;  // unit references index the group's draws
            bp.units = d_units + unit_at;
            bp.counters = d_counters[set];
            bp.large = d_large[set];
            bp.items = d_items[set];
            bp.large_draw = d_large_draw[set];
            bp.count = (uint32_t)n;
            bp.vert_units = (uint32_t)uv.size();
            bp.face_units = (uint32_t)uf.size();
            bp.tile_units = (uint32_t)ut.size();
            bp.clear_units = (uint32_t)uc.size();
            bp.large_cap = large_cap;
            bp.item_cap = item_cap;
            bp.tiles_per_warp = tiles_per_warp;
            if (binned)
                bp.bins = BinSet{d_bin_counters[set],
                                 reinterpret_cast<uint32_t*>(d_bin_counters[set] + 1) + group_bin_at[set], d_crec[set],
                                 (uint32_t)(set_bin_at[set] - group_bin_at[set]), set_crec[set]};
            if (bp.vert_units + bp.face_units + bp.tile_units > 0) b->launches.push_back(L);
        }
    }
    if (async) {
        // through pinned staging, so that the copies are queued without waiting for the work
        // already on the stream
        const size_t tb = sizeof(BatchDraw) * table.size(), ub = sizeof(UnitRef) * units.size();
        const int t = b->stage_next;
        b->stage_next ^= 1;
        if (!b->stage_done[t]) AXR_CUDA(ctx, cudaEventCreateWithFlags(&b->stage_done[t], cudaEventDisableTiming));
        AXR_CUDA(ctx, cudaEventSynchronize(b->stage_done[t]));  // the upload two plans ago has been read
        if (b->stage_bytes[t] < tb + ub) {
            if (b->stage[t]) cudaFreeHost(b->stage[t]);
            b->stage[t] = nullptr;
            b->stage_bytes[t] = 0;
            AXR_CUDA(ctx, cudaMallocHost(&b->stage[t], tb + ub));
            b->stage_bytes[t] = tb + ub;
        }
        unsigned char* h = static_cast<unsigned char*>(b->stage[t]);
        std::memcpy(h, table.data(), tb);
        if (ub) std::memcpy(h + tb, units.data(), ub);
        AXR_CUDA(ctx, cudaMemcpyAsync(d_table, h, tb, cudaMemcpyHostToDevice, ctx->stream));
        if (ub) AXR_CUDA(ctx, cudaMemcpyAsync(d_units, h + tb, ub, cudaMemcpyHostToDevice, ctx->stream));
        AXR_CUDA(ctx, cudaEventRecord(b->stage_done[t], ctx->stream));
    } else {
        AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        AXR_CUDA(ctx, cudaMemcpy(d_table, table.data(), sizeof(BatchDraw) * table.size(), cudaMemcpyHostToDevice));
        if (!units.empty())
            AXR_CUDA(ctx, cudaMemcpy(d_units, units.data(), sizeof(UnitRef) * units.size(), cudaMemcpyHostToDevice));
    }
    b->device = ctx->device;
    b->sets = nsets;
    b->set_counters = d_counters[1];
    b->form = form;
    b->count = (uint32_t)count;
    b->vertices = verts;
    b->faces = faces;
    b->pixels = pixels;
    b->tiles = tiles;
    return AXR_OK;
}

axr_status launch_planned(axr_context* ctx, const axr_batch* b) {
    // a split batch: set 1 on the side stream, forked from and joined back into the context
    // stream (a capture records the same fork and join); with phase timing on, the sets run
    // in turn on the context stream so that each launch's phase events bracket its kernels
    const bool split = b->sets > 1 && !ctx->profile;
    cudaStream_t side = split ? ctx->batch_side.stream : ctx->stream;
    if (split) {
        AXR_CUDA(ctx, cudaEventRecord(ctx->batch_side.fork, ctx->stream));
        AXR_CUDA(ctx, cudaStreamWaitEvent(side, ctx->batch_side.fork, 0));
    }
    for (const axr_batch::Launch& L : b->launches) {
        BatchParams bp = L.params;
        bp.collect_stats = ctx->collect_stats;
        bp.prof = ctx->profile && b->form == kFormPersistent ? ctx->batch_prof : nullptr;
        cudaEvent_t* ev = nullptr;
        if (ctx->profile && b->form != kFormPersistent && !ctx->capturing) {
            while (ctx->batch_events.size() < ctx->batch_events_used + 6) {
                cudaEvent_t e;
                AXR_CUDA(ctx, cudaEventCreate(&e));
                ctx->batch_events.push_back(e);
            }
            ev = &ctx->batch_events[ctx->batch_events_used];
            ctx->batch_events_used += 6;
        }
        // set 1 clears right before its tile pass: its clear (bound by the write rate) then
        // meets set 0's latency-bound tile pass, and set 0's clear meets set 1's vertex and
        // face phases, instead of the two clears meeting each other
        if (b->form == kFormBinned)
            AXR_CUDA(ctx, launch_batch_binned(L.shader, bp, L.set ? side : ctx->stream, ev, &ctx->launches));
        else
            AXR_CUDA(ctx, launch_batch(L.shader, bp, b->form, ctx->cfg.num_sms, L.set ? side : ctx->stream, ev,
                                       &ctx->launches, split && L.set > 0));
    }
    if (b->sets > 1) {
        // set 1's statistics and error bits into the context's counters, which axr_sync and
        // axr_stats_read report
        AXR_CUDA(ctx, launch_merge_counters(ctx->counters, b->set_counters, side));
        ctx->launches += 1;
    }
    if (split) {
        AXR_CUDA(ctx, cudaEventRecord(ctx->batch_side.join, side));
        AXR_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->batch_side.join, 0));
    }
    return AXR_OK;
}

}  // namespace

namespace axr_internal {

axr_status batch_plan(axr_context* ctx, const axr_draw_desc* draws, int32_t count, axr_batch* b, bool async) {
    return plan_batch(ctx, draws, count, b, async);
}

axr_status batch_launch(axr_context* ctx, const axr_batch* b) { return launch_planned(ctx, b); }

void encode_framebuffer_maps(axr_framebuffer* fb) {
    fb->tma = false;
    if (fb->width % 4 != 0) return;  // the row pitch of a tensor map is a multiple of 16 bytes
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return;
    const cuuint64_t dims[2] = {(cuuint64_t)fb->width, (cuuint64_t)fb->height};
    const cuuint64_t pitch[1] = {(cuuint64_t)fb->width * 4};
    const cuuint32_t box[2] = {(cuuint32_t)kTile, (cuuint32_t)kTile};
    const cuuint32_t step[2] = {1, 1};
    const CUresult rc = encode(reinterpret_cast<CUtensorMap*>(&fb->color_map), CU_TENSOR_MAP_DATA_TYPE_UINT32, 2,
                               fb->color, dims, pitch, box, step, CU_TENSOR_MAP_INTERLEAVE_NONE,
                               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const CUresult rd = encode(reinterpret_cast<CUtensorMap*>(&fb->depth_map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                               fb->depth, dims, pitch, box, step, CU_TENSOR_MAP_INTERLEAVE_NONE,
                               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    fb->tma = rc == CUDA_SUCCESS && rd == CUDA_SUCCESS;
}

void mesh_bounds(const float* pos, uint32_t n, float center[3], float* radius) {
    center[0] = center[1] = center[2] = 0.f;
    *radius = 0.f;
    if (!pos || n == 0) return;
    float lo[3] = {pos[0], pos[1], pos[2]}, hi[3] = {pos[0], pos[1], pos[2]};
    for (uint32_t i = 1; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], pos[3ull * i + k]);
            hi[k] = std::max(hi[k], pos[3ull * i + k]);
        }
    for (int k = 0; k < 3; ++k) center[k] = 0.5f * (lo[k] + hi[k]);
    double r2 = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) {
            const double t = (double)pos[3ull * i + k] - center[k];
            s += t * t;
        }
        r2 = std::max(r2, s);
    }
    *radius = (float)std::sqrt(r2) * 1.0001f;
}

void free_batch(axr_batch* b) {
    if (!b) return;
    dfree(b->dev);
    b->dev = nullptr;
    b->bytes = 0;
    b->launches.clear();
}

void free_batch_staging(axr_batch* b) {
    if (!b) return;
    for (int t = 0; t < 2; ++t) {
        if (b->stage_done[t]) {
            cudaEventSynchronize(b->stage_done[t]);
            cudaEventDestroy(b->stage_done[t]);
        }
        if (b->stage[t]) cudaFreeHost(b->stage[t]);
        b->stage[t] = nullptr;
        b->stage_done[t] = nullptr;
        b->stage_bytes[t] = 0;
    }
}

}  // namespace axr_internal

extern "C" {

axr_status axr_batch_create(axr_context* ctx, const axr_draw_desc* draws, int32_t count, axr_batch** out) {
    NvtxRange nvtx_range("axr_batch_create");
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    auto* b = new axr_batch();
    axr_status st = plan_batch(ctx, draws, count, b, false);
    if (st != AXR_OK) {
        free_batch(b);
        delete b;
        return st;
    }
    *out = b;
    return AXR_OK;
}

axr_status axr_batch_launch(axr_context* ctx, axr_batch* b) {
    NvtxRange nvtx_range("axr_batch_launch");
    if (!ctx || !b) return fail(ctx, AXR_E_INVALID, "NULL argument");
    if (b->device != ctx->device) return fail(ctx, AXR_E_INVALID, "batch planned for another device");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    return launch_planned(ctx, b);
}

void axr_batch_destroy(axr_context* ctx, axr_batch* b) {
    if (!b) return;
    DeviceGuard g(b->device);
    if (ctx && ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_batch(b);
    free_batch_staging(b);
    delete b;
}

axr_status axr_batch_get_info(const axr_batch* b, axr_batch_info* out) {
    if (!b || !out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    out->draws = b->count;
    out->launches = (uint32_t)b->launches.size();
    out->form = b->form;
    out->vertices = b->vertices;
    out->faces = b->faces;
    out->pixels = b->pixels;
    out->tiles = b->tiles;
    out->device_bytes = b->bytes;
    return AXR_OK;
}

axr_status axr_draw_batch(axr_context* ctx, const axr_draw_desc* draws, int32_t count) {
    NvtxRange nvtx_range("axr_draw_batch");
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->capturing) return fail(ctx, AXR_E_INVALID, "axr_draw_batch cannot be captured; capture axr_batch_launch");
    DeviceGuard g(ctx->device);
    if (!ctx->oneshot) ctx->oneshot = new axr_batch();
    axr_status st = plan_batch(ctx, draws, count, ctx->oneshot, true);
    if (st != AXR_OK) return st;
    return launch_planned(ctx, ctx->oneshot);
}

int32_t axr_draw_density_class(const axr_draw_desc* draw) { return draw ? density_class(*draw) : 0; }

axr_status axr_batch_get_tuning(const axr_context* ctx, int32_t small_max_pixels[AXR_TUNE_CLASSES]) {
    if (!ctx || !small_max_pixels) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    std::memcpy(small_max_pixels, ctx->tune_small, sizeof(ctx->tune_small));
    return AXR_OK;
}

axr_status axr_batch_set_tuning(axr_context* ctx, const int32_t small_max_pixels[AXR_TUNE_CLASSES]) {
    if (!ctx || !small_max_pixels) return fail(ctx, AXR_E_INVALID, "NULL argument");
    for (int k = 0; k < AXR_TUNE_CLASSES; ++k)
        if (small_max_pixels[k] < 0 || small_max_pixels[k] > 65536)
            return fail(ctx, AXR_E_INVALID, "class %d: pixel box limit %d (0..65536)", k, small_max_pixels[k]);
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::memcpy(ctx->tune_small, small_max_pixels, sizeof(ctx->tune_small));
    return AXR_OK;
}

axr_status axr_batch_get_bin_tuning(const axr_context* ctx, axr_bin_params out[AXR_TUNE_CLASSES]) {
    if (!ctx || !out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    std::memcpy(out, ctx->tune_bin, sizeof(ctx->tune_bin));
    return AXR_OK;
}

axr_status axr_batch_set_bin_tuning(axr_context* ctx, const axr_bin_params params[AXR_TUNE_CLASSES]) {
    if (!ctx || !params) return fail(ctx, AXR_E_INVALID, "NULL argument");
    for (int k = 0; k < AXR_TUNE_CLASSES; ++k)
        if (!valid_bin_params(params[k], false))
            return fail(ctx, AXR_E_INVALID, "class %d: bin parameters (capacity %d: 16..65536, shape %d x %d tiles: 1, "
                        "2, 4 or 8 each with at most 8 in all, thread pixels %d: 1..2048)", k, params[k].capacity,
                        params[k].tiles_x, params[k].tiles_y, params[k].thread_pixels);
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::memcpy(ctx->tune_bin, params, sizeof(ctx->tune_bin));
    return AXR_OK;
}

axr_status axr_batch_autotune(axr_context* ctx, const axr_draw_desc* draws, int32_t count, int32_t repeats,
                              int32_t out_small_max_pixels[AXR_TUNE_CLASSES]) {
    NvtxRange nvtx_range("axr_batch_autotune");
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    if (repeats < 1) repeats = 1;
    axr_status st = check_draws(ctx, draws, count);
    if (st != AXR_OK) return st;
    static const int32_t kCandidates[] = {16, 32, 64, 128, 256};
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->capturing) return fail(ctx, AXR_E_INVALID, "cannot tune during graph capture");
    DeviceGuard g(ctx->device);
    std::vector<std::vector<axr_draw_desc>> by_class(AXR_TUNE_CLASSES);
    for (int32_t i = 0; i < count; ++i) by_class[(size_t)density_class(draws[i])].push_back(draws[i]);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    AXR_CUDA(ctx, cudaEventCreate(&e0));
    AXR_CUDA(ctx, cudaEventCreate(&e1));
    axr_batch trial;
    st = AXR_OK;
    // time `sub` as planned now: warm-up launch, then `repeats` launches between events
    auto time_plan = [&](const axr_draw_desc* sub, int32_t n, float* ms) -> axr_status {
        axr_status r = plan_batch(ctx, sub, n, &trial, false);
        if (r != AXR_OK) return r;
        if ((r = launch_planned(ctx, &trial)) != AXR_OK) return r;
        cudaError_t e = cudaEventRecord(e0, ctx->stream);
        for (int32_t i = 0; i < repeats && e == cudaSuccess && r == AXR_OK; ++i) r = launch_planned(ctx, &trial);
        if (r != AXR_OK) return r;
        if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
        return e == cudaSuccess ? AXR_OK : cuda_fail(ctx, e, "autotune timing");
    };
    // the binned form's bin parameters per density class, by coordinate descent on the
    // sub-batch of that class: per-thread raster limit, then bin shape, then capacity
    {
        const int saved_form = ctx->batch_form;
        ctx->batch_form = kFormBinned;
        static const int32_t kThreadPx[] = {1, 4, 8, 16, 32, 64, 128, 256};
        static const int32_t kShapes[][2] = {{8, 1}, {4, 2}, {2, 4}, {4, 1}, {2, 2}, {2, 1}, {1, 1}};
        static const int32_t kCapacity[] = {64, 128, 256, 512, 1024, 2048};
        for (int k = 0; k < AXR_TUNE_CLASSES && st == AXR_OK; ++k) {
            const std::vector<axr_draw_desc>& sub = by_class[(size_t)k];
            if (sub.empty()) continue;
            auto descend = [&](int32_t axr_bin_params::*field, const int32_t* cands, size_t n) {
                float best_ms = 0.f;
                int32_t best = ctx->tune_bin[k].*field;
                for (size_t c = 0; c < n && st == AXR_OK; ++c) {
                    ctx->tune_bin[k].*field = cands[c];
                    float ms = 0.f;
                    if ((st = time_plan(sub.data(), (int32_t)sub.size(), &ms)) != AXR_OK) break;
                    if (best_ms == 0.f || ms < best_ms) {
                        best_ms = ms;
                        best = cands[c];
                    }
                }
                ctx->tune_bin[k].*field = best;
            };
            descend(&axr_bin_params::thread_pixels, kThreadPx, sizeof(kThreadPx) / sizeof(kThreadPx[0]));
            {  // bin shape: tiles across and down together
                float best_ms = 0.f;
                axr_bin_params best = ctx->tune_bin[k];
                for (const auto& sh : kShapes) {
                    if (st != AXR_OK) break;
                    ctx->tune_bin[k].tiles_x = sh[0];
                    ctx->tune_bin[k].tiles_y = sh[1];
                    float ms = 0.f;
                    if ((st = time_plan(sub.data(), (int32_t)sub.size(), &ms)) != AXR_OK) break;
                    if (best_ms == 0.f || ms < best_ms) {
                        best_ms = ms;
                        best = ctx->tune_bin[k];
                    }
                }
                ctx->tune_bin[k] = best;
            }
            descend(&axr_bin_params::capacity, kCapacity, sizeof(kCapacity) / sizeof(kCapacity[0]));
        }
        ctx->batch_form = saved_form;
    }
    // launch form: the three forms on the whole batch
    if (st == AXR_OK) {
        float best_ms = 0.f;
        int best = ctx->batch_form;
        for (int form : {kFormPersistent, kFormPhased, kFormBinned}) {
            ctx->batch_form = form;
            float ms = 0.f;
            if ((st = time_plan(draws, count, &ms)) != AXR_OK) break;
            if (best_ms == 0.f || ms < best_ms) {
                best_ms = ms;
                best = form;
            }
        }
        ctx->batch_form = best;
    }
    // the keyed forms' per-thread pixel-box limit per density class
    for (int k = 0; k < AXR_TUNE_CLASSES && st == AXR_OK && ctx->batch_form != kFormBinned; ++k) {
        const std::vector<axr_draw_desc>& sub = by_class[(size_t)k];
        if (sub.empty()) continue;
        float best_ms = 0.f;
        int32_t best = ctx->tune_small[k];
        for (int32_t cand : kCandidates) {
            ctx->tune_small[k] = cand;
            float ms = 0.f;
            if ((st = time_plan(sub.data(), (int32_t)sub.size(), &ms)) != AXR_OK) break;
            if (best_ms == 0.f || ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
        ctx->tune_small[k] = best;
    }
    cudaStreamSynchronize(ctx->stream);
    free_batch(&trial);
    free_batch_staging(&trial);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != AXR_OK) return st;
    if (out_small_max_pixels) std::memcpy(out_small_max_pixels, ctx->tune_small, sizeof(ctx->tune_small));
    return AXR_OK;
}

axr_status axr_batch_set_form(axr_context* ctx, int32_t form) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    if (form != AXR_BATCH_PERSISTENT && form != AXR_BATCH_PHASED && form != AXR_BATCH_BINNED)
        return fail(ctx, AXR_E_INVALID, "unknown batch launch form %d", form);
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->batch_form = form;
    return AXR_OK;
}

int32_t axr_batch_get_form(const axr_context* ctx) { return ctx ? ctx->batch_form : -1; }

}  // extern "C"
