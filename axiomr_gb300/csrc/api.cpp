// C ABI implementation (include/axr.h): contexts, device resources, per-draw uniforms
// and launch orchestration. The draw kernels are in kernels.cu; this file only plans
// and enqueues work on the context's stream.
#include "axr.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device_types.h"
#include "hostmath.h"
#include "kernels.h"

using namespace axr;

#include "api_types.h"
#include "api_internal.h"
#include "batch.h"

namespace axr_internal {

thread_local std::string g_no_ctx_error;

axr_status fail(axr_context* ctx, axr_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx)
        ctx->error = buf;
    else
        g_no_ctx_error = buf;
    return st;
}

axr_status cuda_fail(axr_context* ctx, cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(ctx, AXR_E_OOM, "%s: out of device memory", what);
    }
    return fail(ctx, AXR_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void dfree(void* p) {
    if (p) cudaFree(p);
}

// Whether no vertex of the mesh can lie outside or on any of the six clip planes
// (x+w, w-x, y+w, w-y, z+w, w-z >= 0 of clip = mvp * (p, 1)) for the column-major mvp: the
// smallest value of each plane's function over the mesh's bounding sphere, in double, must
// exceed a margin far above the rounding of the device's float evaluation. Unknown bounds
// (an update still in flight) or non-finite values answer false.
bool mesh_clip_free(const axr_mesh* m, const float mvp[16]) {
    if (!m || m->num_vertices == 0) return false;
    if (m->bounds_pending) {
        if (cudaEventQuery(m->bounds_ready) != cudaSuccess) {
            cudaGetLastError();  // cudaErrorNotReady is no error here
            return false;
        }
        mesh_sync_bounds(m);
        if (m->bounds_pending) return false;
    }
    const double c[3] = {m->bound_center[0], m->bound_center[1], m->bound_center[2]};
    const double r = m->bound_radius;
    const double extent = std::max({std::fabs(c[0]), std::fabs(c[1]), std::fabs(c[2])}) + r + 1.0;
    for (int k = 0; k < 6; ++k) {
        const int j = k / 2;                       // the x, y or z row of the matrix
        const double s = (k % 2 == 0) ? 1.0 : -1.0;  // w + row or w - row
        double g[3], norm2 = 0.0, terms = 0.0;
        for (int i = 0; i < 3; ++i) {
            g[i] = (double)mvp[4 * i + 3] + s * (double)mvp[4 * i + j];
            norm2 += g[i] * g[i];
        }
        const double h = (double)mvp[12 + 3] + s * (double)mvp[12 + j];
        for (int i = 0; i < 4; ++i) terms += std::fabs((double)mvp[4 * i + 3]) + std::fabs((double)mvp[4 * i + j]);
        const double lowest = g[0] * c[0] + g[1] * c[1] + g[2] * c[2] + h - r * std::sqrt(norm2);
        if (!(lowest > 1e-5 * terms * extent)) return false;
    }
    return true;
}

void mesh_sync_bounds(const axr_mesh* m) {
    static std::mutex mu;  // planners on several threads may share a mesh
    if (!m) return;
    std::lock_guard<std::mutex> lk(mu);
    if (!m->bounds_pending) return;
    if (cudaEventSynchronize(m->bounds_ready) != cudaSuccess) return;  // keep the previous bounds
    const MeshBounds& b = *m->bounds_host;
    for (int k = 0; k < 3; ++k)
        m->bound_center[k] = 0.5f * (mesh_bounds_float(b.lo[k]) + mesh_bounds_float(b.hi[k]));
    double r2;
    std::memcpy(&r2, &b.r2, sizeof(r2));
    m->bound_radius = m->num_vertices ? (float)std::sqrt(r2) * 1.0001f : 0.f;
    m->bounds_pending = false;
}

}  // namespace axr_internal

using namespace axr_internal;

namespace {

DevTexture dev_texture(const axr_texture* t) {
    DevTexture d{};
    if (t) {
        d.texels = t->texels;
        d.width = t->width;
        d.height = t->height;
    }
    return d;
}

void free_scratch(axr_context* ctx) {
    dfree(ctx->large);
    dfree(ctx->items);
    dfree(ctx->vscreen);
    dfree(ctx->vattr);
    dfree(ctx->shade);
    dfree(ctx->clip_px);
    dfree(ctx->rec);
    ctx->large = nullptr;
    ctx->items = nullptr;
    ctx->vscreen = ctx->vattr = nullptr;
    ctx->shade = ctx->clip_px = nullptr;
    ctx->rec = nullptr;
    ctx->large_cap = ctx->item_cap = ctx->vcap = ctx->px_cap = ctx->rec_cap = 0;
}

void free_bins(axr_context* ctx) {
    dfree(ctx->bin_mem);
    dfree(ctx->bin_entries);
    dfree(ctx->bin_crec);
    ctx->bin_mem = nullptr;
    ctx->bin_entries = nullptr;
    ctx->bin_crec = nullptr;
    ctx->bin_count_cap = ctx->crec_cap = 0;
    ctx->bin_entry_cap = 0;
}

axr_status grow_scratch(axr_context* ctx, uint32_t faces, uint32_t vertices, uint64_t pixels) {
    // Large-triangle setups and tile work items (a triangle that finds either list full is
    // rasterised by its own thread instead, so those two sizes trade memory for speed), the
    // per-vertex cache of the vertex pass (one entry per vertex) and the clipped-winner
    // pixel list (at most one entry per pixel).
    uint32_t want_tris = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(65536, (uint64_t)faces), 1u << 25);
    uint32_t want_items = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(1u << 20, 4ull * faces), 1u << 27);
    uint32_t want_verts = std::max<uint32_t>(4096, vertices);
    uint32_t want_px = (uint32_t)std::max<uint64_t>(1u << 16, pixels);
    uint32_t want_rec = std::max<uint32_t>(4096, faces);  // one shading record per face
    if (want_tris <= ctx->large_cap && want_items <= ctx->item_cap && want_verts <= ctx->vcap &&
        want_px <= ctx->px_cap && want_rec <= ctx->rec_cap)
        return AXR_OK;
    if (ctx->capturing)
        return fail(ctx, AXR_E_CAPACITY, "scratch for %u faces / %u vertices not reserved before graph capture",
                    faces, vertices);
    want_tris = std::max(want_tris, ctx->large_cap);
    want_items = std::max(want_items, ctx->item_cap);
    want_verts = std::max(want_verts, ctx->vcap);
    want_px = std::max(want_px, ctx->px_cap);
    want_rec = std::max(want_rec, ctx->rec_cap);
    AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    free_scratch(ctx);
    AXR_CUDA(ctx, dmalloc(&ctx->large, want_tris));
    AXR_CUDA(ctx, dmalloc(&ctx->items, want_items));
    AXR_CUDA(ctx, dmalloc(&ctx->vscreen, want_verts));
    AXR_CUDA(ctx, dmalloc(&ctx->vattr, 4ull * want_verts));
    AXR_CUDA(ctx, dmalloc(&ctx->shade, want_px));
    AXR_CUDA(ctx, dmalloc(&ctx->clip_px, want_px));
    AXR_CUDA(ctx, dmalloc(&ctx->rec, (size_t)kRecFloat4 * want_rec));
    ctx->rec_cap = want_rec;
    ctx->large_cap = want_tris;
    ctx->item_cap = want_items;
    ctx->vcap = want_verts;
    ctx->px_cap = want_px;
    return AXR_OK;
}

axr_status check_mesh_desc(axr_context* ctx, const axr_mesh_desc* d) {
    if (!d) return fail(ctx, AXR_E_INVALID, "mesh descriptor is NULL");
    if (d->num_vertices && (!d->positions || !d->uvs || !d->normals))
        return fail(ctx, AXR_E_INVALID, "mesh needs positions, uvs and normals");
    if (d->num_faces && !d->indices) return fail(ctx, AXR_E_INVALID, "mesh has faces but no indices");
    if (d->num_groups && !d->groups) return fail(ctx, AXR_E_INVALID, "mesh has groups but no group array");
    if (d->num_materials && !d->materials) return fail(ctx, AXR_E_INVALID, "mesh has materials but no array");
    uint64_t drawn = 0;
    for (uint32_t g = 0; g < d->num_groups; ++g) {
        const axr_group_desc& gr = d->groups[g];
        if ((uint64_t)gr.start_face + gr.face_count > d->num_faces)
            return fail(ctx, AXR_E_INVALID, "group %u covers faces beyond the mesh", g);
        if (gr.material >= d->num_materials)
            return fail(ctx, AXR_E_INVALID, "group %u names material %u of %u", g, gr.material, d->num_materials);
        drawn += gr.face_count;
    }
    if (drawn > kMaxOrdinal + 1ull)
        return fail(ctx, AXR_E_CAPACITY, "a draw is limited to %u faces", kMaxOrdinal + 1u);
    for (uint64_t i = 0; i < 3ull * d->num_faces; ++i)
        if (d->indices[i] >= d->num_vertices)
            return fail(ctx, AXR_E_INVALID, "face %llu indexes vertex %u of %u", (unsigned long long)(i / 3),
                        d->indices[i], d->num_vertices);
    return AXR_OK;
}

// Upload float3 arrays via the staging buffer and widen them to float4.
axr_status upload_vec3(axr_context* ctx, axr_mesh* m, const float* src, float4* dst) {
    if (!src || !dst || m->num_vertices == 0) return AXR_OK;
    AXR_CUDA(ctx, cudaMemcpyAsync(m->staging, src, 12ull * m->num_vertices, cudaMemcpyHostToDevice, ctx->stream));
    AXR_CUDA(ctx, launch_pack3(m->staging, dst, m->num_vertices, ctx->stream));
    ++ctx->launches;
    return AXR_OK;
}

axr_status upload_mesh_arrays(axr_context* ctx, axr_mesh* m, const axr_mesh_desc* d) {
    axr_status st;
    if ((st = upload_vec3(ctx, m, d->positions, m->pos)) != AXR_OK) return st;
    if ((st = upload_vec3(ctx, m, d->normals, m->nrm)) != AXR_OK) return st;
    if ((st = upload_vec3(ctx, m, d->tangents, m->tan)) != AXR_OK) return st;
    if ((st = upload_vec3(ctx, m, d->bitangents, m->bit)) != AXR_OK) return st;
    if (m->num_vertices)
        AXR_CUDA(ctx, cudaMemcpyAsync(m->uv, d->uvs, 8ull * m->num_vertices, cudaMemcpyHostToDevice, ctx->stream));
    if (m->num_faces)
        AXR_CUDA(ctx, cudaMemcpyAsync(m->idx, d->indices, 12ull * m->num_faces, cudaMemcpyHostToDevice, ctx->stream));
    return AXR_OK;
}

void free_mesh(axr_mesh* m) {
    if (!m) return;
    dfree(m->pos); dfree(m->nrm); dfree(m->tan); dfree(m->bit); dfree(m->uv); dfree(m->idx);
    dfree(m->groups); dfree(m->materials); dfree(m->staging); dfree(m->bounds_dev);
    if (m->bounds_ready) {
        cudaEventSynchronize(m->bounds_ready);
        cudaEventDestroy(m->bounds_ready);
    }
    if (m->bounds_host) cudaFreeHost(m->bounds_host);
    delete m;
}

// Scratch of the binned per-draw form: bin counters and counts for `bins` bins, `entries`
// bin entries and `crec` clipped-triangle records (grown, never shrunk).
axr_status grow_bins(axr_context* ctx, uint32_t bins, size_t entries, uint32_t crec) {
    if (bins <= ctx->bin_count_cap && entries <= ctx->bin_entry_cap && crec <= ctx->crec_cap) return AXR_OK;
    if (ctx->capturing)
        return fail(ctx, AXR_E_CAPACITY,
                    "bin scratch for %u bins / %zu entries / %u clipped records not reserved before graph capture "
                    "(reserved %u / %zu / %u)", bins, entries, crec, ctx->bin_count_cap, ctx->bin_entry_cap,
                    ctx->crec_cap);
    bins = std::max(bins, ctx->bin_count_cap);
    entries = std::max(entries, ctx->bin_entry_cap);
    crec = std::max(crec, ctx->crec_cap);
    AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    free_bins(ctx);
    AXR_CUDA(ctx, cudaMalloc(&ctx->bin_mem, sizeof(BinCounters) + sizeof(uint32_t) * (size_t)bins));
    AXR_CUDA(ctx, dmalloc(&ctx->bin_entries, entries));
    AXR_CUDA(ctx, dmalloc(&ctx->bin_crec, (size_t)kRasterRec * crec));
    ctx->bin_count_cap = bins;
    ctx->bin_entry_cap = entries;
    ctx->crec_cap = crec;
    return AXR_OK;
}

// Bin shape and capacity of a binned draw of `faces` faces into `fb`.
struct BinPlan {
    uint16_t bins_x, bins_y;
    uint8_t tw, th;
    uint32_t cap, crec;
    uint32_t bins() const { return (uint32_t)bins_x * bins_y; }
};

BinPlan plan_bins(const axr_bin_params& bp, const axr_framebuffer* fb, uint32_t faces) {
    BinPlan b{};
    if (bp.tiles_x > 0) {
        bin_shape(bp, &b.tw, &b.th);
    } else {  // about 2,400 or more bins (16 per SM of a GB300), 1 to 8 tiles each
        const uint32_t tiles = (uint32_t)fb->tiles_x * (uint32_t)fb->tiles_y;
        uint32_t nt = 1;
        while (nt < 8 && tiles / (2 * nt) >= 2432) nt *= 2;
        b.tw = (uint8_t)(nt >= 2 ? 2 : 1) * (uint8_t)(nt == 8 ? 2 : 1);
        b.th = (uint8_t)(nt / b.tw);
    }
    bin_geometry(fb->tiles_x, fb->tiles_y, b.tw, b.th, &b.bins_x, &b.bins_y);
    if (bp.capacity > 0) {
        b.cap = (uint32_t)bp.capacity;
    } else {  // twice the mean entries per bin, a power of two in [64, 16384]; the entries of
              // a denser bin spill through the key plane, which spreads them over all threads
        const uint64_t mean = 2ull * faces / std::max<uint32_t>(1, b.bins());
        uint32_t c = 64;
        while (c < mean && c < 16384) c <<= 1;
        b.cap = c;
    }
    b.crec = std::max<uint32_t>(1u << 16, faces / 4);
    return b;
}

DrawParams make_params(axr_context* ctx, const axr_mesh* m, const axr_framebuffer* fb, const DevUniforms& u) {
    DrawParams p{};
    p.mesh = DevMesh{m->pos, m->nrm, m->tan, m->bit, m->uv, m->idx, m->groups, m->materials,
                     m->num_vertices, m->num_faces, m->num_groups, m->num_drawn};
    p.target = DevTarget{fb->color, fb->depth, fb->key, fb->tile_flag,
                         fb->width, fb->height, fb->tiles_x, fb->tiles_y};
    p.u = u;
    p.scratch = DevScratch{ctx->counters, ctx->large, ctx->items, ctx->vscreen, ctx->vattr,
                           ctx->shade, ctx->clip_px, ctx->large_cap, ctx->item_cap, ctx->vcap, ctx->px_cap,
                           ctx->collect_stats, 0, nullptr, ctx->rec};
    p.small_max_pixels = ctx->small_max_pixels;
    return p;
}

bool valid_kind(int32_t k) { return k >= AXR_SHADER_FLAT && k <= AXR_SHADER_GOURAUD; }

}  // namespace

extern "C" {

axr_status axr_context_create(int32_t device, axr_context** out) {
    if (!out) return fail(nullptr, AXR_E_INVALID, "out is NULL");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(nullptr, AXR_E_UNSUPPORTED, "no CUDA device available");
    }
    if (device < 0 || device >= n) return fail(nullptr, AXR_E_INVALID, "device %d of %d", device, n);
    DeviceGuard g(device);
    auto* ctx = new axr_context();
    ctx->device = device;
    cudaDeviceProp prop{};
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e == cudaSuccess && prop.major < 10) {
        delete ctx;
        return fail(nullptr, AXR_E_UNSUPPORTED, "device %d is sm_%d%d; this build targets sm_103a", device,
                    prop.major, prop.minor);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    // the side stream runs work that fills gaps beside the main stream's (the clipped-winner
    // pass, the batched form's clears): lowest priority, so the main stream's CTAs go first
    int prio_low = 0, prio_high = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ctx->aux.stream, cudaStreamNonBlocking, prio_low);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->aux.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->aux.join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->batch_side.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->batch_side.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->batch_side.join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->counters, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMemset(ctx->counters, 0, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->batch_prof, sizeof(BatchProfile));
    if (e == cudaSuccess) e = cudaMemset(ctx->batch_prof, 0, sizeof(BatchProfile));
    if (e != cudaSuccess) {
        axr_status st = cuda_fail(nullptr, e, "context setup");
        if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
        if (ctx->aux.stream) cudaStreamDestroy(ctx->aux.stream);
        if (ctx->aux.fork) cudaEventDestroy(ctx->aux.fork);
        if (ctx->aux.join) cudaEventDestroy(ctx->aux.join);
        if (ctx->batch_side.stream) cudaStreamDestroy(ctx->batch_side.stream);
        if (ctx->batch_side.fork) cudaEventDestroy(ctx->batch_side.fork);
        if (ctx->batch_side.join) cudaEventDestroy(ctx->batch_side.join);
        dfree(ctx->counters);
        dfree(ctx->batch_prof);
        delete ctx;
        return st;
    }
    ctx->stream = ctx->own_stream;
    ctx->cfg.num_sms = prop.multiProcessorCount;
    ctx->cfg.large_ctas_per_sm = 2;
    ctx->cfg.resolve_ctas_per_sm = 4;
    *out = ctx;
    return AXR_OK;
}

void axr_context_destroy(axr_context* ctx) {
    if (!ctx) return;
    DeviceGuard g(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (cudaEvent_t ev : ctx->event_pool) cudaEventDestroy(ev);
    for (cudaEvent_t ev : ctx->batch_events) cudaEventDestroy(ev);
    if (ctx->oneshot) {
        free_batch(ctx->oneshot);
        free_batch_staging(ctx->oneshot);
        delete ctx->oneshot;
    }
    dfree(ctx->counters);
    dfree(ctx->batch_prof);
    free_scratch(ctx);
    free_bins(ctx);
    free_png(ctx);
    if (ctx->aux.stream) cudaStreamSynchronize(ctx->aux.stream);
    if (ctx->aux.stream) cudaStreamDestroy(ctx->aux.stream);
    for (int k = 0; k < axr_context::kCopyStreams; ++k) {
        if (ctx->copy_stream[k]) {
            cudaStreamSynchronize(ctx->copy_stream[k]);
            cudaStreamDestroy(ctx->copy_stream[k]);
        }
        if (ctx->copy_join[k]) cudaEventDestroy(ctx->copy_join[k]);
    }
    if (ctx->copy_fork) cudaEventDestroy(ctx->copy_fork);
    if (ctx->aux.fork) cudaEventDestroy(ctx->aux.fork);
    if (ctx->aux.join) cudaEventDestroy(ctx->aux.join);
    if (ctx->batch_side.stream) {
        cudaStreamSynchronize(ctx->batch_side.stream);
        cudaStreamDestroy(ctx->batch_side.stream);
    }
    if (ctx->batch_side.fork) cudaEventDestroy(ctx->batch_side.fork);
    if (ctx->batch_side.join) cudaEventDestroy(ctx->batch_side.join);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

int32_t axr_abi_version(void) { return AXR_ABI_VERSION; }

axr_status axr_diag_barrier_timeout(axr_context* ctx, uint32_t timeout_ms) {
    if (!ctx || timeout_ms == 0 || timeout_ms > 10000) return fail(ctx, AXR_E_INVALID, "timeout_ms must be 1..10000");
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        DeviceGuard g(ctx->device);
        AXR_CUDA(ctx, launch_barrier_probe(ctx->counters, (unsigned long long)timeout_ms * 1000000ull, ctx->stream));
        ctx->launches += 1;
    }
    return axr_sync(ctx);
}

const char* axr_last_error(const axr_context* ctx) { return ctx ? ctx->error.c_str() : g_no_ctx_error.c_str(); }

void* axr_context_stream(axr_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

axr_status axr_context_set_stream(axr_context* ctx, void* stream) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return AXR_OK;
}

axr_status axr_sync(axr_context* ctx) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t err = 0;
    AXR_CUDA(ctx, cudaMemcpy(&err, &ctx->counters->error, sizeof(err), cudaMemcpyDeviceToHost));
    if (err) {
        AXR_CUDA(ctx, cudaMemset(&ctx->counters->error, 0, sizeof(uint32_t)));
        if (err & kErrBarrier)
            return fail(ctx, AXR_E_TIMEOUT, "a grid barrier of the batched kernel timed out (error bits 0x%x)", err);
        if (err & kErrTma)
            return fail(ctx, AXR_E_TIMEOUT, "a tile load of the binned form did not arrive (error bits 0x%x)", err);
        return fail(ctx, AXR_E_CAPACITY, "device reported error bits 0x%x", err);
    }
    return AXR_OK;
}

axr_status axr_reserve(axr_context* ctx, uint32_t max_faces) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    axr_status st = grow_scratch(ctx, max_faces, max_faces * 3u, 3840ull * 2160ull);
    if (st != AXR_OK) return st;
    // the binned form's bins for a 3840x2160 framebuffer in the smallest-bin shape
    axr_framebuffer probe{};
    probe.tiles_x = (3840 + kTile - 1) / kTile;
    probe.tiles_y = (2160 + kTile - 1) / kTile;
    // at most one bin per tile; a sized-per-draw capacity is a power of two below
    // 4 * faces / bins (at least 64), so bins * capacity stays below max(64 * bins, 4 * faces)
    const uint32_t bins = (uint32_t)probe.tiles_x * (uint32_t)probe.tiles_y;
    const size_t entries = ctx->bin_params.capacity > 0 ? (size_t)bins * (size_t)ctx->bin_params.capacity
                                                        : std::max<size_t>(64ull * bins, 4ull * max_faces);
    return grow_bins(ctx, bins, entries, std::max<uint32_t>(1u << 16, max_faces / 4));
}

void* axr_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void axr_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

// ---------------------------------------------------------------- textures
axr_status axr_texture_create(axr_context* ctx, const uint8_t* rgba, int32_t width, int32_t height,
                              axr_texture** out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    *out = nullptr;
    if (width <= 0 || height <= 0 || !rgba) return fail(ctx, AXR_E_INVALID, "texture %dx%d", width, height);
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    auto* t = new axr_texture();
    t->width = width;
    t->height = height;
    t->device = ctx->device;
    size_t n = (size_t)width * (size_t)height;
    cudaError_t e = dmalloc(&t->texels, n);
    if (e == cudaSuccess) e = cudaMemcpy(t->texels, rgba, n * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        dfree(t->texels);
        delete t;
        return cuda_fail(ctx, e, "texture upload");
    }
    *out = t;
    return AXR_OK;
}

axr_status axr_texture_update(axr_context* ctx, axr_texture* t, const uint8_t* rgba) {
    if (!ctx || !t || !rgba) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, cudaMemcpyAsync(t->texels, rgba, (size_t)t->width * t->height * 4, cudaMemcpyHostToDevice,
                                  ctx->stream));
    return AXR_OK;
}

void axr_texture_destroy(axr_context* ctx, axr_texture* t) {
    if (!t) return;
    DeviceGuard g(t->device);
    if (ctx && ctx->stream) cudaStreamSynchronize(ctx->stream);
    dfree(t->texels);
    delete t;
}

// ---------------------------------------------------------------- meshes
axr_status axr_mesh_create(axr_context* ctx, const axr_mesh_desc* d, axr_mesh** out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    *out = nullptr;
    axr_status st = check_mesh_desc(ctx, d);
    if (st != AXR_OK) return st;
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    auto* m = new axr_mesh();
    m->device = ctx->device;
    m->num_vertices = d->num_vertices;
    m->num_faces = d->num_faces;
    m->num_groups = d->num_groups;
    m->num_materials = d->num_materials;
    const uint32_t V = d->num_vertices;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto** p, size_t n) {
        if (e == cudaSuccess) e = dmalloc(p, n);
    };
    alloc(&m->pos, V);
    alloc(&m->nrm, V);
    alloc(&m->uv, V);
    if (d->tangents) alloc(&m->tan, V);
    if (d->bitangents) alloc(&m->bit, V);
    alloc(&m->idx, 3ull * d->num_faces);
    alloc(&m->staging, 3ull * V);
    alloc(&m->groups, std::max<uint32_t>(1, d->num_groups));
    alloc(&m->materials, std::max<uint32_t>(1, d->num_materials));
    if (e != cudaSuccess) {
        free_mesh(m);
        return cuda_fail(ctx, e, "mesh allocation");
    }
    std::vector<DevGroup> groups(std::max<uint32_t>(1, d->num_groups));
    uint32_t base = 0;
    for (uint32_t k = 0; k < d->num_groups; ++k) {
        groups[k] = DevGroup{d->groups[k].start_face, d->groups[k].face_count, base, d->groups[k].material};
        base += d->groups[k].face_count;
    }
    m->num_drawn = base;
    mesh_bounds(d->positions, V, m->bound_center, &m->bound_radius);
    std::vector<DevMaterial> mats(std::max<uint32_t>(1, d->num_materials));
    for (uint32_t k = 0; k < d->num_materials; ++k) {
        const axr_material_desc& md = d->materials[k];
        DevMaterial& dm = mats[k];
        dm = DevMaterial{};
        dm.diffuse = dev_texture(md.diffuse);
        dm.bump = dev_texture(md.bump);
        dm.metallic = dev_texture(md.metallic);
        dm.roughness = dev_texture(md.roughness);
        dm.ao = dev_texture(md.ao);
        dm.specular_exponent = md.specular_exponent;
    }
    st = upload_mesh_arrays(ctx, m, d);
    if (st == AXR_OK) {
        e = cudaMemcpyAsync(m->groups, groups.data(), groups.size() * sizeof(DevGroup), cudaMemcpyHostToDevice,
                            ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(m->materials, mats.data(), mats.size() * sizeof(DevMaterial),
                                cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "mesh upload");
    }
    if (st != AXR_OK) {
        free_mesh(m);
        return st;
    }
    *out = m;
    return AXR_OK;
}

// Above this many vertices axr_mesh_update computes the bounds on the device (five small
// stream operations cost about as much as a host pass over 8k vertices).
constexpr uint32_t kHostBoundsMaxVertices = 8192;

axr_status axr_mesh_update(axr_context* ctx, axr_mesh* m, const axr_mesh_desc* d) {
    if (!ctx || !m || !d) return fail(ctx, AXR_E_INVALID, "NULL argument");
    if (d->num_vertices != m->num_vertices || d->num_faces != m->num_faces)
        return fail(ctx, AXR_E_INVALID, "mesh update must keep vertex and face counts");
    if ((d->tangents && !m->tan) || (d->bitangents && !m->bit))
        return fail(ctx, AXR_E_INVALID, "mesh was created without tangents/bitangents");
    if (d->num_vertices && (!d->positions || !d->uvs || !d->normals))
        return fail(ctx, AXR_E_INVALID, "mesh update needs positions, uvs and normals");
    if (d->num_faces && !d->indices) return fail(ctx, AXR_E_INVALID, "mesh update needs indices");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    axr_status st = upload_mesh_arrays(ctx, m, d);
    if (st != AXR_OK) return st;
    // the bounding sphere of the new positions: a host pass for a small mesh (a few us);
    // for a large one on the device behind the upload (a host pass over a million vertices
    // takes milliseconds), which batch planning waits for if it must
    if (m->num_vertices <= kHostBoundsMaxVertices) {
        mesh_bounds(d->positions, d->num_vertices, m->bound_center, &m->bound_radius);
        m->bounds_pending = false;
        return AXR_OK;
    }
    if (!m->bounds_dev) {
        AXR_CUDA(ctx, cudaMalloc(&m->bounds_dev, sizeof(MeshBounds)));
        AXR_CUDA(ctx, cudaMallocHost(&m->bounds_host, sizeof(MeshBounds)));
        AXR_CUDA(ctx, cudaEventCreateWithFlags(&m->bounds_ready, cudaEventDisableTiming));
    }
    AXR_CUDA(ctx, launch_mesh_bounds(m->pos, m->num_vertices, m->bounds_dev, ctx->stream));
    AXR_CUDA(ctx, cudaMemcpyAsync(m->bounds_host, m->bounds_dev, sizeof(MeshBounds), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    AXR_CUDA(ctx, cudaEventRecord(m->bounds_ready, ctx->stream));
    m->bounds_pending = true;
    ctx->launches += m->num_vertices ? 2 : 0;
    return AXR_OK;
}

void axr_mesh_destroy(axr_context* ctx, axr_mesh* m) {
    if (!m) return;
    DeviceGuard g(m->device);
    if (ctx && ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_mesh(m);
}

// ---------------------------------------------------------------- framebuffers
axr_status axr_framebuffer_create(axr_context* ctx, int32_t width, int32_t height, axr_framebuffer** out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    *out = nullptr;
    if (width <= 0 || height <= 0 || width > 32768 || height > 32768)
        return fail(ctx, AXR_E_INVALID, "framebuffer %dx%d (1..32768 per side)", width, height);
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    auto* fb = new axr_framebuffer();
    fb->width = width;
    fb->height = height;
    fb->tiles_x = (width + kTile - 1) / kTile;
    fb->tiles_y = (height + kTile - 1) / kTile;
    fb->device = ctx->device;
    size_t n = (size_t)width * height, nt = (size_t)fb->tiles_x * fb->tiles_y;
    cudaError_t e = dmalloc(&fb->color, n);
    if (e == cudaSuccess) e = dmalloc(&fb->depth, n);
    if (e == cudaSuccess) e = dmalloc(&fb->key, n);
    if (e == cudaSuccess) e = dmalloc(&fb->tile_flag, nt);
    if (e == cudaSuccess) e = cudaMemsetAsync(fb->tile_flag, 0, nt * 4, ctx->stream);
    if (e == cudaSuccess) e = launch_fill_u64(fb->key, n, kEmptyKey, ctx->stream);
    // Framebuffer(w, h, true): colour 0, depth +inf (src/framebuffer.cpp:6-14)
    if (e == cudaSuccess) e = launch_clear(fb->color, fb->depth, n, 0u, INFINITY, true, true, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        dfree(fb->color); dfree(fb->depth); dfree(fb->key); dfree(fb->tile_flag);
        delete fb;
        return cuda_fail(ctx, e, "framebuffer allocation");
    }
    encode_framebuffer_maps(fb);
    *out = fb;
    return AXR_OK;
}

void axr_framebuffer_destroy(axr_context* ctx, axr_framebuffer* fb) {
    if (!fb) return;
    DeviceGuard g(fb->device);
    if (ctx && ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx && ctx->fb == fb) ctx->fb = nullptr;
    dfree(fb->color); dfree(fb->depth); dfree(fb->key); dfree(fb->tile_flag);
    delete fb;
}

axr_status axr_framebuffer_clear_color(axr_context* ctx, axr_framebuffer* fb, uint8_t r, uint8_t g_, uint8_t b,
                                       uint8_t a) {
    if (!ctx || !fb) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    // packed a<<24 | r<<16 | g<<8 | b, i.e. bytes B, G, R, A (src/framebuffer.cpp:26-36)
    uint32_t packed = ((uint32_t)a << 24) | ((uint32_t)r << 16) | ((uint32_t)g_ << 8) | (uint32_t)b;
    AXR_CUDA(ctx, launch_clear(fb->color, nullptr, (size_t)fb->width * fb->height, packed, 0.f, true, false,
                               ctx->stream));
    ++ctx->launches;
    return AXR_OK;
}

axr_status axr_framebuffer_clear_depth(axr_context* ctx, axr_framebuffer* fb, float depth) {
    if (!ctx || !fb) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, launch_clear(nullptr, fb->depth, (size_t)fb->width * fb->height, 0u, depth, false, true,
                               ctx->stream));
    ++ctx->launches;
    return AXR_OK;
}

static axr_status fb_read(axr_context* ctx, const axr_framebuffer* fb, uint8_t* bgra, float* depth, bool wait) {
    if (!ctx || !fb) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    size_t n = (size_t)fb->width * fb->height;
    if (bgra) AXR_CUDA(ctx, cudaMemcpyAsync(bgra, fb->color, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (depth) AXR_CUDA(ctx, cudaMemcpyAsync(depth, fb->depth, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (wait) AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return AXR_OK;
}

axr_status axr_framebuffer_read(axr_context* ctx, const axr_framebuffer* fb, uint8_t* bgra, float* depth) {
    return fb_read(ctx, fb, bgra, depth, true);
}

axr_status axr_framebuffers_read_async(axr_context* ctx, int32_t count, const axr_framebuffer* const* fbs,
                                       uint8_t* const* bgra, float* const* depth) {
    if (!ctx || count < 0 || (count > 0 && !fbs)) return fail(ctx, AXR_E_INVALID, "bad framebuffer list");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    if (!ctx->copy_fork) {
        AXR_CUDA(ctx, cudaEventCreateWithFlags(&ctx->copy_fork, cudaEventDisableTiming));
        for (int k = 0; k < axr_context::kCopyStreams; ++k) {
            AXR_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream[k], cudaStreamNonBlocking));
            AXR_CUDA(ctx, cudaEventCreateWithFlags(&ctx->copy_join[k], cudaEventDisableTiming));
        }
    }
    // the copies start after the work already enqueued on the context stream, and the
    // context stream continues after all of them
    AXR_CUDA(ctx, cudaEventRecord(ctx->copy_fork, ctx->stream));
    for (int k = 0; k < axr_context::kCopyStreams; ++k) AXR_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream[k], ctx->copy_fork, 0));
    for (int32_t i = 0; i < count; ++i) {
        const axr_framebuffer* fb = fbs[i];
        if (!fb) return fail(ctx, AXR_E_INVALID, "framebuffer %d is NULL", i);
        const size_t n = (size_t)fb->width * fb->height;
        cudaStream_t st = ctx->copy_stream[i % axr_context::kCopyStreams];
        if (bgra && bgra[i]) AXR_CUDA(ctx, cudaMemcpyAsync(bgra[i], fb->color, n * 4, cudaMemcpyDeviceToHost, st));
        if (depth && depth[i]) AXR_CUDA(ctx, cudaMemcpyAsync(depth[i], fb->depth, n * 4, cudaMemcpyDeviceToHost, st));
    }
    for (int k = 0; k < axr_context::kCopyStreams; ++k) {
        AXR_CUDA(ctx, cudaEventRecord(ctx->copy_join[k], ctx->copy_stream[k]));
        AXR_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copy_join[k], 0));
    }
    return AXR_OK;
}

axr_status axr_framebuffer_read_async(axr_context* ctx, const axr_framebuffer* fb, uint8_t* bgra, float* depth) {
    return fb_read(ctx, fb, bgra, depth, false);
}

}  // extern "C"

// A read-back on its own copy streams: started after the work already on the context
// stream, but later work on the context stream does not wait for it.
struct axr_readback {
    int device = 0;
    static constexpr int kStreams = 4;
    cudaStream_t copy[kStreams] = {};
    cudaEvent_t copied[kStreams] = {};
    cudaEvent_t ready = nullptr;  // the framebuffers are final (context stream)
    // packed read-backs: the gathered planes on the device and the plane table
    uint8_t* staging = nullptr;
    size_t staging_cap = 0;
    axr::PackedImage* images = nullptr;       // device
    axr::PackedImage* images_host = nullptr;  // pinned
    uint32_t images_cap = 0;
};

namespace {

void release_readback(axr_readback* rb) {
    for (int k = 0; k < axr_readback::kStreams; ++k) {
        if (rb->copy[k]) {
            cudaStreamSynchronize(rb->copy[k]);
            cudaStreamDestroy(rb->copy[k]);
        }
        if (rb->copied[k]) cudaEventDestroy(rb->copied[k]);
    }
    if (rb->ready) cudaEventDestroy(rb->ready);
    dfree(rb->staging);
    dfree(rb->images);
    if (rb->images_host) cudaFreeHost(rb->images_host);
    delete rb;
}

}  // namespace

extern "C" {

axr_status axr_readback_create(axr_context* ctx, axr_readback** out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    DeviceGuard g(ctx->device);
    auto* rb = new axr_readback();
    rb->device = ctx->device;
    cudaError_t e = cudaEventCreateWithFlags(&rb->ready, cudaEventDisableTiming);
    for (int k = 0; e == cudaSuccess && k < axr_readback::kStreams; ++k) {
        e = cudaStreamCreateWithFlags(&rb->copy[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&rb->copied[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        release_readback(rb);
        return cuda_fail(ctx, e, "read-back streams");
    }
    *out = rb;
    return AXR_OK;
}

void axr_readback_destroy(axr_context* ctx, axr_readback* rb) {
    if (!rb) return;
    DeviceGuard g(rb->device);
    release_readback(rb);
}

axr_status axr_readback_start(axr_context* ctx, axr_readback* rb, int32_t count, const axr_framebuffer* const* fbs,
                              uint8_t* const* bgra, float* const* depth) {
    NvtxRange nvtx_range("axr_readback_start");
    if (!ctx || !rb || count < 0 || (count > 0 && !fbs)) return fail(ctx, AXR_E_INVALID, "bad read-back arguments");
    if (rb->device != ctx->device) return fail(ctx, AXR_E_INVALID, "the read-back belongs to another device");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, cudaEventRecord(rb->ready, ctx->stream));
    for (int k = 0; k < axr_readback::kStreams; ++k) AXR_CUDA(ctx, cudaStreamWaitEvent(rb->copy[k], rb->ready, 0));
    for (int32_t i = 0; i < count; ++i) {
        const axr_framebuffer* fb = fbs[i];
        if (!fb) return fail(ctx, AXR_E_INVALID, "framebuffer %d is NULL", i);
        const size_t n = (size_t)fb->width * fb->height;
        cudaStream_t st = rb->copy[i % axr_readback::kStreams];
        if (bgra && bgra[i]) AXR_CUDA(ctx, cudaMemcpyAsync(bgra[i], fb->color, n * 4, cudaMemcpyDeviceToHost, st));
        if (depth && depth[i]) AXR_CUDA(ctx, cudaMemcpyAsync(depth[i], fb->depth, n * 4, cudaMemcpyDeviceToHost, st));
    }
    for (int k = 0; k < axr_readback::kStreams; ++k) AXR_CUDA(ctx, cudaEventRecord(rb->copied[k], rb->copy[k]));
    return AXR_OK;
}

axr_status axr_readback_start_packed(axr_context* ctx, axr_readback* rb, int32_t count,
                                     const axr_framebuffer* const* fbs, int32_t format, uint8_t* host,
                                     uint64_t capacity) {
    NvtxRange nvtx_range("axr_readback_start_packed");
    if (!ctx || !rb || count < 0 || (count > 0 && (!fbs || !host))) return fail(ctx, AXR_E_INVALID, "bad read-back arguments");
    if (format != AXR_PACKED_BGRA && format != AXR_PACKED_RGB) return fail(ctx, AXR_E_INVALID, "unknown format %d", format);
    if (rb->device != ctx->device) return fail(ctx, AXR_E_INVALID, "the read-back belongs to another device");
    const uint32_t bpp = format == AXR_PACKED_RGB ? 3u : 4u;
    uint64_t bytes = 0, pixels = 0;
    for (int32_t i = 0; i < count; ++i) {
        if (!fbs[i]) return fail(ctx, AXR_E_INVALID, "framebuffer %d is NULL", i);
        pixels += (uint64_t)fbs[i]->width * fbs[i]->height;
    }
    bytes = pixels * bpp;
    if (capacity < bytes)
        return fail(ctx, AXR_E_INVALID, "the host buffer holds %llu bytes, the images need %llu",
                    (unsigned long long)capacity, (unsigned long long)bytes);
    if (count == 0) return AXR_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    // the previous read-back of this object has finished with its staging and table
    for (int k = 0; k < axr_readback::kStreams; ++k) AXR_CUDA(ctx, cudaEventSynchronize(rb->copied[k]));
    if (bytes > rb->staging_cap) {
        dfree(rb->staging);
        rb->staging = nullptr;
        rb->staging_cap = 0;
        AXR_CUDA(ctx, dmalloc(&rb->staging, (size_t)bytes));
        rb->staging_cap = (size_t)bytes;
    }
    if ((uint32_t)count > rb->images_cap) {
        dfree(rb->images);
        rb->images = nullptr;
        if (rb->images_host) cudaFreeHost(rb->images_host);
        rb->images_host = nullptr;
        rb->images_cap = 0;
        AXR_CUDA(ctx, dmalloc(&rb->images, (size_t)count));
        AXR_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&rb->images_host), sizeof(axr::PackedImage) * count));
        rb->images_cap = (uint32_t)count;
    }
    uint64_t first = 0;
    for (int32_t i = 0; i < count; ++i) {
        const axr_framebuffer* fb = fbs[i];
        rb->images_host[i] = axr::PackedImage{fb->color, first * bpp, (uint32_t)fb->width, (uint32_t)fb->height, first};
        first += (uint64_t)fb->width * fb->height;
    }
    // gather on the context stream behind the frames, then the copies on the read-back's
    // streams; later work on the context stream does not wait for the copies
    AXR_CUDA(ctx, cudaMemcpyAsync(rb->images, rb->images_host, sizeof(axr::PackedImage) * count,
                                  cudaMemcpyHostToDevice, ctx->stream));
    AXR_CUDA(ctx, launch_packed(rb->images, (uint32_t)count, pixels, format == AXR_PACKED_RGB, rb->staging,
                                ctx->cfg.num_sms, ctx->stream));
    ctx->launches += 1;
    AXR_CUDA(ctx, cudaEventRecord(rb->ready, ctx->stream));
    const uint64_t part = (bytes + axr_readback::kStreams - 1) / axr_readback::kStreams;
    for (int k = 0; k < axr_readback::kStreams; ++k) {
        AXR_CUDA(ctx, cudaStreamWaitEvent(rb->copy[k], rb->ready, 0));
        const uint64_t lo = std::min<uint64_t>(bytes, part * k), hi = std::min<uint64_t>(bytes, lo + part);
        if (hi > lo)
            AXR_CUDA(ctx, cudaMemcpyAsync(host + lo, rb->staging + lo, hi - lo, cudaMemcpyDeviceToHost, rb->copy[k]));
        AXR_CUDA(ctx, cudaEventRecord(rb->copied[k], rb->copy[k]));
    }
    return AXR_OK;
}

axr_status axr_readback_wait(axr_context* ctx, axr_readback* rb) {
    if (!rb) return fail(ctx, AXR_E_INVALID, "NULL argument");
    DeviceGuard g(rb->device);
    for (int k = 0; k < axr_readback::kStreams; ++k) AXR_CUDA(ctx, cudaEventSynchronize(rb->copied[k]));
    return AXR_OK;
}

axr_status axr_framebuffer_write(axr_context* ctx, axr_framebuffer* fb, const uint8_t* bgra, const float* depth) {
    if (!ctx || !fb) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    size_t n = (size_t)fb->width * fb->height;
    if (bgra) AXR_CUDA(ctx, cudaMemcpyAsync(fb->color, bgra, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    if (depth) AXR_CUDA(ctx, cudaMemcpyAsync(fb->depth, depth, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return AXR_OK;
}

axr_status axr_framebuffer_size(const axr_framebuffer* fb, int32_t* width, int32_t* height) {
    if (!fb) return fail(nullptr, AXR_E_INVALID, "framebuffer is NULL");
    if (width) *width = fb->width;
    if (height) *height = fb->height;
    return AXR_OK;
}

axr_status axr_framebuffer_device_pointers(const axr_framebuffer* fb, void** bgra, void** depth) {
    if (!fb) return fail(nullptr, AXR_E_INVALID, "framebuffer is NULL");
    if (bgra) *bgra = fb->color;
    if (depth) *depth = fb->depth;
    return AXR_OK;
}

// ---------------------------------------------------------------- pipeline state and draws
axr_status axr_set_shader(axr_context* ctx, const axr_shader_desc* s) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!s) {
        ctx->has_shader = false;
        return AXR_OK;
    }
    if (!valid_kind(s->kind)) return fail(ctx, AXR_E_INVALID, "unknown shader kind %d", s->kind);
    ctx->shader = *s;
    ctx->has_shader = true;
    return AXR_OK;
}

axr_status axr_set_camera(axr_context* ctx, const axr_camera_desc* c) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!c) {
        ctx->has_camera = false;
        return AXR_OK;
    }
    ctx->camera = *c;
    ctx->has_camera = true;
    return AXR_OK;
}

axr_status axr_set_framebuffer(axr_context* ctx, axr_framebuffer* fb) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->fb = fb;
    return AXR_OK;
}

axr_status axr_draw_mesh(axr_context* ctx, const axr_mesh* mesh, const float model[16]) {
    NvtxRange nvtx_range("axr_draw_mesh");
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    if (!mesh || !model) return fail(ctx, AXR_E_INVALID, "NULL mesh or model matrix");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->has_shader || !ctx->has_camera || !ctx->fb) return AXR_OK;  // src/tiled_pipeline.cpp:146
    DeviceGuard g(ctx->device);
    axr_status st = grow_scratch(ctx, mesh->num_drawn, mesh->num_vertices,
                                 (uint64_t)ctx->fb->width * (uint64_t)ctx->fb->height);
    if (st != AXR_OK) return st;
    DevUniforms u = make_uniforms(ctx->camera, ctx->shader, model);
    DrawParams p = make_params(ctx, mesh, ctx->fb, u);
    BinPlan bp{};
    if (ctx->draw_form == AXR_DRAW_BINNED) {
        bp = plan_bins(ctx->bin_params, ctx->fb, mesh->num_drawn);
        st = grow_bins(ctx, bp.bins(), (size_t)bp.bins() * bp.cap, bp.crec);
        if (st != AXR_OK) return st;
    }
    cudaEvent_t* ev = nullptr;
    if (ctx->profile && !ctx->capturing) {
        while (ctx->event_pool.size() < ctx->events_used + kStageEvents) {
            cudaEvent_t e;
            AXR_CUDA(ctx, cudaEventCreate(&e));
            ctx->event_pool.push_back(e);
        }
        ev = &ctx->event_pool[ctx->events_used];
        ctx->events_used += kStageEvents;
    }
    if (ctx->draw_form != AXR_DRAW_BINNED) {
        LaunchConfig cfg = ctx->cfg;
        cfg.clip_free = mesh_clip_free(mesh, u.mvp);
        AXR_CUDA(ctx, launch_draw(p, cfg, ctx->stream, &ctx->aux, ev, &ctx->launches));
        return AXR_OK;
    }
    SoloBinned sb{};
    sb.color_map = ctx->fb->color_map;
    sb.depth_map = ctx->fb->depth_map;
    sb.p = p;
    sb.p.bins = DevBins{ctx->bin_entries, 0u, bp.cap, bp.bins_x, bp.bins_y, bp.tw, bp.th,
                        (uint16_t)ctx->bin_params.thread_pixels};
    sb.bins = BinSet{ctx->bin_mem, reinterpret_cast<uint32_t*>(ctx->bin_mem + 1), ctx->bin_crec, bp.bins(),
                     ctx->crec_cap};
    sb.flags = ctx->fb->tma ? kBatchTma : 0u;
    AXR_CUDA(ctx, launch_draw_binned(sb, ctx->stream, ev, &ctx->launches));
    return AXR_OK;
}

axr_status axr_set_draw_form(axr_context* ctx, int32_t form) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    if (form != AXR_DRAW_BINNED && form != AXR_DRAW_KEYED) return fail(ctx, AXR_E_INVALID, "unknown draw form %d", form);
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->draw_form = form;
    return AXR_OK;
}

int32_t axr_get_draw_form(const axr_context* ctx) { return ctx ? ctx->draw_form : -1; }

axr_status axr_set_bin_params(axr_context* ctx, const axr_bin_params* params) {
    if (!ctx || !params) return fail(ctx, AXR_E_INVALID, "NULL argument");
    if (!valid_bin_params(*params, true))
        return fail(ctx, AXR_E_INVALID, "bin parameters: capacity %d (0 or 16..65536), shape %d x %d tiles (0, or 1, 2, "
                    "4 or 8 each with at most 8 in all), thread pixels %d (1..2048)", params->capacity, params->tiles_x,
                    params->tiles_y, params->thread_pixels);
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->bin_params = *params;
    return AXR_OK;
}

axr_status axr_get_bin_params(const axr_context* ctx, axr_bin_params* out) {
    if (!ctx || !out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    *out = ctx->bin_params;
    return AXR_OK;
}

// ---------------------------------------------------------------- graphs
axr_status axr_graph_begin(axr_context* ctx) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->capturing) return fail(ctx, AXR_E_INVALID, "capture already active");
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = true;
    return AXR_OK;
}

axr_status axr_graph_end(axr_context* ctx, axr_graph** out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->capturing) return fail(ctx, AXR_E_INVALID, "no capture active");
    DeviceGuard g(ctx->device);
    ctx->capturing = false;
    cudaGraph_t graph = nullptr;
    AXR_CUDA(ctx, cudaStreamEndCapture(ctx->stream, &graph));
    auto* gr = new axr_graph();
    gr->device = ctx->device;
    cudaError_t e = cudaGraphInstantiate(&gr->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        delete gr;
        return cuda_fail(ctx, e, "graph instantiate");
    }
    *out = gr;
    return AXR_OK;
}

axr_status axr_graph_launch(axr_context* ctx, axr_graph* gr) {
    if (!ctx || !gr) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, cudaGraphLaunch(gr->exec, ctx->stream));
    return AXR_OK;
}

void axr_graph_destroy(axr_graph* gr) {
    if (!gr) return;
    DeviceGuard g(gr->device);
    if (gr->exec) cudaGraphExecDestroy(gr->exec);
    delete gr;
}

// ---------------------------------------------------------------- camera helpers
axr_status axr_camera_matrices(const float position[3], const float target[3], float fov_degrees, float aspect,
                               float view[16], float projection[16], float view_proj[16]) {
    if (!position || !target) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    host::M4 v, p, vp;
    host::camera_matrices(position, target, fov_degrees, aspect, v, p, vp);
    if (view) std::memcpy(view, v.m, sizeof(v.m));
    if (projection) std::memcpy(projection, p.m, sizeof(p.m));
    if (view_proj) std::memcpy(view_proj, vp.m, sizeof(vp.m));
    return AXR_OK;
}

axr_status axr_viewport_matrix(int32_t x, int32_t y, int32_t width, int32_t height, float out[16]) {
    if (!out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    host::M4 v = host::viewport_matrix(x, y, width, height);
    std::memcpy(out, v.m, sizeof(v.m));
    return AXR_OK;
}

// ---------------------------------------------------------------- statistics
axr_status axr_stats_enable(axr_context* ctx, int32_t enable) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->collect_stats = enable ? 1 : 0;
    return AXR_OK;
}

axr_status axr_stats_read(axr_context* ctx, axr_draw_stats* out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    DevCounters c{};
    AXR_CUDA(ctx, cudaMemcpy(&c, ctx->counters, sizeof(c), cudaMemcpyDeviceToHost));
    out->triangles = c.stat_triangles;
    out->fragments = c.stat_fragments;
    out->large = c.stat_large;
    out->tiles = c.stat_tiles;
    out->tested = c.stat_tested;
    out->shaded = c.stat_shaded;
    AXR_CUDA(ctx, cudaMemset(&ctx->counters->stat_triangles, 0, 6 * sizeof(unsigned long long)));
    return AXR_OK;
}

// ---------------------------------------------------------------- profiling
axr_status axr_profile_enable(axr_context* ctx, int32_t enable) {
    if (!ctx) return fail(nullptr, AXR_E_INVALID, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->profile = enable != 0;
    return AXR_OK;
}

axr_status axr_profile_read(axr_context* ctx, axr_profile* out) {
    if (!ctx || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    axr_profile r{};
    for (size_t k = 0; k + kStageEvents <= ctx->events_used; k += kStageEvents) {
        double* out[6] = {&r.vertex_ms, &r.geometry_ms, &r.large_ms, &r.scan_ms, &r.shade_ms, &r.clipped_ms};
        for (int j = 0; j < 6; ++j) {
            float ms = 0.f;
            AXR_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->event_pool[k + j], ctx->event_pool[k + j + 1]));
            *out[j] += ms;
        }
        ++r.draws;
    }
    ctx->events_used = 0;
    BatchProfile bp{};
    AXR_CUDA(ctx, cudaMemcpy(&bp, ctx->batch_prof, sizeof(bp), cudaMemcpyDeviceToHost));
    AXR_CUDA(ctx, cudaMemset(ctx->batch_prof, 0, sizeof(bp.phase_ns) + sizeof(bp.launches)));
    r.batch_launches = bp.launches;
    r.batch_vertex_ms = bp.phase_ns[0] * 1e-6;
    r.batch_face_ms = bp.phase_ns[1] * 1e-6;
    r.batch_large_ms = bp.phase_ns[2] * 1e-6;
    r.batch_tile_ms = bp.phase_ns[3] * 1e-6;
    for (size_t k = 0; k + 6 <= ctx->batch_events_used; k += 6) {
        double* out[5] = {&r.batch_clear_ms, &r.batch_vertex_ms, &r.batch_face_ms, &r.batch_large_ms,
                          &r.batch_tile_ms};
        for (int j = 0; j < 5; ++j) {
            float ms = 0.f;
            AXR_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->batch_events[k + j], ctx->batch_events[k + j + 1]));
            *out[j] += ms;
        }
        ++r.batch_launches;
    }
    ctx->batch_events_used = 0;
    r.kernel_launches = ctx->launches;
    *out = r;
    return AXR_OK;
}

// ---------------------------------------------------------------- stage access
axr_status axr_debug_triangles(axr_context* ctx, const axr_mesh* mesh, const float model[16],
                               const float view_proj[16], int32_t width, int32_t height, float* out,
                               uint32_t capacity, uint32_t* count) {
    if (!ctx || !mesh || !model || !view_proj || !count) return fail(ctx, AXR_E_INVALID, "NULL argument");
    if (width <= 0 || height <= 0) return fail(ctx, AXR_E_INVALID, "target %dx%d", width, height);
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    axr_camera_desc cam{};
    std::memcpy(cam.view_proj, view_proj, sizeof(cam.view_proj));
    axr_shader_desc sh{};
    sh.kind = AXR_SHADER_GOURAUD;
    DevUniforms u = make_uniforms(cam, sh, model);
    axr_framebuffer fake{};
    fake.width = width;
    fake.height = height;
    DrawParams p = make_params(ctx, mesh, &fake, u);
    float* d_out = nullptr;
    uint32_t* d_count = nullptr;
    cudaError_t e = dmalloc(&d_out, 14ull * std::max<uint32_t>(1, capacity));
    if (e == cudaSuccess) e = dmalloc(&d_count, 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_count, 0, 4, ctx->stream);
    if (e == cudaSuccess) e = launch_debug_triangles(p, d_out, d_count, capacity, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(count, d_count, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess && out)
        e = cudaMemcpy(out, d_out, 14ull * 4 * std::min(*count, capacity), cudaMemcpyDeviceToHost);
    dfree(d_out);
    dfree(d_count);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "debug triangles");
    return AXR_OK;
}

axr_status axr_debug_sample(axr_context* ctx, const axr_texture* tex, const float* uv, int32_t n, float* out) {
    if (!ctx || !tex || !uv || !out || n < 0) return fail(ctx, AXR_E_INVALID, "bad argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    float2* d_uv = nullptr;
    float4* d_out = nullptr;
    cudaError_t e = dmalloc(&d_uv, std::max(1, n));
    if (e == cudaSuccess) e = dmalloc(&d_out, std::max(1, n));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_uv, uv, 8ull * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = launch_debug_sample(dev_texture(tex), d_uv, d_out, (uint32_t)n, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, 16ull * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(d_uv);
    dfree(d_out);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "debug sample");
    return AXR_OK;
}

}  // extern "C"
