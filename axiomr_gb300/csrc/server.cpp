// Serving loop (include/axr.h, "serving loop"): a host thread that admits render requests
// against a device-memory budget and renders whatever has arrived as one batch while the
// previous batch's read-backs are still in flight (continuous batching).
//
// Per iteration the worker (1) retires batches whose read-backs finished (request done,
// framebuffer back to its pool, assets unpinned), (2) if a batch slot is free, admits
// queued requests in arrival order until the batch is full or the next request does not
// fit: its mesh and textures are made resident (uploaded on the upload stream from pinned
// host copies, the least recently used unpinned assets and idle framebuffers evicted when
// the budget would be exceeded) and a framebuffer of its size is taken from the pool,
// (3) launches the admitted group (draw table upload + batched kernels on the context
// stream, behind the upload event) and enqueues each request's read-back on the copy
// stream behind the kernel, then (4) waits briefly for new requests or completions.
// Device memory is allocated and freed stream-ordered (cudaMallocAsync / cudaFreeAsync), so
// growth and eviction never synchronise the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "api_internal.h"
#include "api_types.h"

using namespace axr;
using namespace axr_internal;

namespace {

uint64_t steady_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// Pinned host copy of an array (source of asynchronous uploads).
struct HostBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~HostBuf() {
        if (p) cudaFreeHost(p);
    }
    bool assign(const void* src, size_t n) {
        bytes = n;
        if (n == 0) return true;
        if (cudaHostAlloc(&p, n, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return false;
        }
        std::memcpy(p, src, n);
        return true;
    }
};

struct TexAsset {
    HostBuf rgba;
    int32_t width = 0, height = 0;
    axr_texture dev{};   // texels == nullptr when not resident
    uint64_t last_use = 0;
    int pins = 0;
    size_t bytes() const { return (size_t)width * (size_t)height * 4; }
};

struct MeshAsset {
    uint32_t nv = 0, nf = 0, num_drawn = 0;
    HostBuf pos, nrm, tan, bit, uv, idx;  // pos/nrm/tan/bit widened to float4 on the host
    std::vector<DevGroup> groups;
    std::vector<axr_server_material> mats;
    std::vector<int32_t> textures;        // distinct texture ids of the materials
    float bound_center[3] = {0, 0, 0};
    float bound_radius = 0;
    axr_mesh dev{};                       // pos == nullptr when not resident
    uint64_t mat_gen = 0;                 // texture generation the material table was built for
    uint64_t last_use = 0;
    int pins = 0;
    size_t bytes() const {
        return pos.bytes + nrm.bytes + tan.bytes + bit.bytes + uv.bytes + idx.bytes +
               sizeof(DevGroup) * std::max<size_t>(1, groups.size()) + sizeof(DevMaterial) * std::max<size_t>(1, mats.size());
    }
};

struct Fb {
    axr_framebuffer fb{};
    bool busy = false;
    uint64_t last_use = 0;
    size_t bytes() const {
        const size_t n = (size_t)fb.width * (size_t)fb.height;
        return n * (4 + 4 + 8) + (size_t)fb.tiles_x * (size_t)fb.tiles_y * 4;
    }
};

struct Req {
    axr_server_request r{};
    uint64_t arrival = 0, launch = 0, done = 0, batch_id = 0;
    uint32_t batch_size = 0;
    int status = AXR_OK;
    int png_status = AXR_OK;  // the PNG file did not fit its buffer, or the encode failed
    uint64_t png_bytes = 0;
    bool finished = false;
    Fb* fb = nullptr;
};

struct Slot {
    // with overlap_kernels, the slot's own context: its stream, work counters and draw
    // scratch, so that the kernels of batches in different slots run side by side;
    // otherwise null and the slot renders on the server's context
    axr_context* sctx = nullptr;
    axr_batch plan;
    std::vector<Req*> reqs;
    cudaEvent_t kernel_done = nullptr, copies_done = nullptr;
    // PNG outputs: the RGB and RGBA files of the slot's requests, encoded right after the
    // batch on the context stream; their copies are issued on the copy stream once the
    // encode is done (its sizes are then known), behind the raw read-backs
    axr_png_batch* png[2] = {};
    std::vector<Req*> png_reqs[2];
    cudaEvent_t files_done = nullptr;
    bool files_pending = false, files_issued = false;
    bool busy = false;
    uint64_t id = 0;
};

}  // namespace

struct axr_server {
    axr_server_config cfg{};
    axr_context* ctx = nullptr;
    cudaStream_t upload = nullptr, copy = nullptr;
    cudaEvent_t uploaded = nullptr;
    cudaEvent_t home_ready = nullptr;  // the home stream's allocations and frees so far
    std::vector<std::unique_ptr<TexAsset>> textures;
    std::vector<std::unique_ptr<MeshAsset>> meshes;
    std::vector<std::unique_ptr<Fb>> fbs;
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
    uint64_t next_ticket = 1, tick = 0, next_batch = 1, tex_gen = 1;
    bool stop = false;
    bool hold = false;
    std::thread worker;
    axr_server_stats stats{};
    uint64_t resident = 0;
    std::string error;

    // ---------------------------------------------------------------- memory
    void account(int64_t delta) {
        resident = (uint64_t)((int64_t)resident + delta);
        stats.resident_bytes = resident;
        stats.peak_bytes = std::max(stats.peak_bytes, resident);
    }

    void evict_texture(TexAsset& t) {
        cudaFreeAsync(const_cast<uint32_t*>(t.dev.texels), ctx->stream);
        t.dev.texels = nullptr;
        account(-(int64_t)t.bytes());
        ++tex_gen;  // material tables naming it are stale
        ++stats.evictions;
    }

    void free_mesh_arrays(axr_mesh& m) {
        void* ps[] = {m.pos, m.nrm, m.tan, m.bit, m.uv, m.idx, m.groups, m.materials};
        for (void* p : ps)
            if (p) cudaFreeAsync(p, ctx->stream);
        m = axr_mesh{};
    }

    void evict_mesh(MeshAsset& m) {
        free_mesh_arrays(m.dev);
        account(-(int64_t)m.bytes());
        ++stats.evictions;
    }

    void free_fb(Fb& f) {
        void* ps[] = {f.fb.color, f.fb.depth, f.fb.key, f.fb.tile_flag};
        for (void* p : ps)
            if (p) cudaFreeAsync(p, ctx->stream);
        account(-(int64_t)f.bytes());
    }

    // Evict the least recently used unpinned asset or idle framebuffer; false if none.
    bool evict_one() {
        uint64_t best = UINT64_MAX;
        int kind = -1;
        size_t at = 0;
        for (size_t i = 0; i < meshes.size(); ++i)
            if (meshes[i]->dev.pos && meshes[i]->pins == 0 && meshes[i]->last_use < best) {
                best = meshes[i]->last_use;
                kind = 0;
                at = i;
            }
        for (size_t i = 0; i < textures.size(); ++i)
            if (textures[i]->dev.texels && textures[i]->pins == 0 && textures[i]->last_use < best) {
                best = textures[i]->last_use;
                kind = 1;
                at = i;
            }
        for (size_t i = 0; i < fbs.size(); ++i)
            if (!fbs[i]->busy && fbs[i]->last_use < best) {
                best = fbs[i]->last_use;
                kind = 2;
                at = i;
            }
        if (kind == 0) evict_mesh(*meshes[at]);
        if (kind == 1) evict_texture(*textures[at]);
        if (kind == 2) {
            free_fb(*fbs[at]);
            fbs.erase(fbs.begin() + (ptrdiff_t)at);
        }
        return kind >= 0;
    }

    bool make_room(uint64_t need) {
        while (resident + need > cfg.memory_budget_bytes)
            if (!evict_one()) return false;
        return true;
    }

    // ---------------------------------------------------------------- residency
    cudaError_t upload_texture(TexAsset& t) {
        void* p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, t.bytes(), upload);
        if (e == cudaSuccess) e = cudaMemcpyAsync(p, t.rgba.p, t.bytes(), cudaMemcpyHostToDevice, upload);
        if (e != cudaSuccess) return e;
        t.dev.texels = static_cast<uint32_t*>(p);
        t.dev.width = t.width;
        t.dev.height = t.height;
        t.dev.device = ctx->device;
        account((int64_t)t.bytes());
        ++stats.uploads;
        return cudaSuccess;
    }

    cudaError_t upload_materials(MeshAsset& m) {
        std::vector<DevMaterial> dm(std::max<size_t>(1, m.mats.size()));
        auto view = [&](int32_t id) {
            DevTexture d{};
            if (id >= 0) {
                const TexAsset& t = *textures[(size_t)id];
                d.texels = t.dev.texels;
                d.width = t.width;
                d.height = t.height;
            }
            return d;
        };
        for (size_t k = 0; k < m.mats.size(); ++k) {
            const axr_server_material& sm = m.mats[k];
            dm[k] = DevMaterial{};
            dm[k].diffuse = view(sm.diffuse);
            dm[k].bump = view(sm.bump);
            dm[k].metallic = view(sm.metallic);
            dm[k].roughness = view(sm.roughness);
            dm[k].ao = view(sm.ao);
            dm[k].specular_exponent = sm.specular_exponent;
        }
        // pageable source: the copy is staged before cudaMemcpyAsync returns
        cudaError_t e = cudaMemcpyAsync(m.dev.materials, dm.data(), sizeof(DevMaterial) * dm.size(),
                                        cudaMemcpyHostToDevice, upload);
        m.mat_gen = tex_gen;
        return e;
    }

    cudaError_t upload_mesh(MeshAsset& m) {
        axr_mesh& d = m.dev;
        cudaError_t e = cudaSuccess;
        auto put = [&](auto** dst, const HostBuf& src) {
            if (e != cudaSuccess || src.bytes == 0) return;
            void* p = nullptr;
            e = cudaMallocAsync(&p, src.bytes, upload);
            if (e == cudaSuccess) e = cudaMemcpyAsync(p, src.p, src.bytes, cudaMemcpyHostToDevice, upload);
            *dst = static_cast<std::remove_pointer_t<decltype(dst)>>(p);
        };
        put(&d.pos, m.pos);
        put(&d.nrm, m.nrm);
        put(&d.tan, m.tan);
        put(&d.bit, m.bit);
        put(&d.uv, m.uv);
        put(&d.idx, m.idx);
        void* g = nullptr;
        void* mt = nullptr;
        if (e == cudaSuccess) e = cudaMallocAsync(&g, sizeof(DevGroup) * std::max<size_t>(1, m.groups.size()), upload);
        if (e == cudaSuccess && !m.groups.empty())
            e = cudaMemcpyAsync(g, m.groups.data(), sizeof(DevGroup) * m.groups.size(), cudaMemcpyHostToDevice, upload);
        if (e == cudaSuccess) e = cudaMallocAsync(&mt, sizeof(DevMaterial) * std::max<size_t>(1, m.mats.size()), upload);
        d.groups = static_cast<DevGroup*>(g);
        d.materials = static_cast<DevMaterial*>(mt);
        d.num_vertices = m.nv;
        d.num_faces = m.nf;
        d.num_groups = (uint32_t)m.groups.size();
        d.num_materials = (uint32_t)m.mats.size();
        d.num_drawn = m.num_drawn;
        d.device = ctx->device;
        std::memcpy(d.bound_center, m.bound_center, sizeof(d.bound_center));
        d.bound_radius = m.bound_radius;
        if (e == cudaSuccess) e = upload_materials(m);
        if (e != cudaSuccess) return e;
        account((int64_t)m.bytes());
        ++stats.uploads;
        return cudaSuccess;
    }

    cudaError_t new_framebuffer(int32_t w, int32_t h, Fb** out) {
        auto f = std::make_unique<Fb>();
        axr_framebuffer& fb = f->fb;
        fb.width = w;
        fb.height = h;
        fb.tiles_x = (w + kTile - 1) / kTile;
        fb.tiles_y = (h + kTile - 1) / kTile;
        fb.device = ctx->device;
        const size_t n = (size_t)w * (size_t)h, nt = (size_t)fb.tiles_x * fb.tiles_y;
        void *c = nullptr, *d = nullptr, *k = nullptr, *t = nullptr;
        cudaError_t e = cudaMallocAsync(&c, n * 4, ctx->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&d, n * 4, ctx->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&k, n * 8, ctx->stream);
        if (e == cudaSuccess) e = cudaMallocAsync(&t, nt * 4, ctx->stream);
        fb.color = static_cast<uint32_t*>(c);
        fb.depth = static_cast<float*>(d);
        fb.key = static_cast<unsigned long long*>(k);
        fb.tile_flag = static_cast<uint32_t*>(t);
        if (e == cudaSuccess) e = cudaMemsetAsync(fb.tile_flag, 0, nt * 4, ctx->stream);
        if (e == cudaSuccess) e = launch_fill_u64(fb.key, n, kEmptyKey, ctx->stream);
        if (e != cudaSuccess) {
            free_fb(*f);
            return e;
        }
        encode_framebuffer_maps(&fb);
        account((int64_t)f->bytes());
        ++stats.framebuffers;
        *out = f.get();
        fbs.push_back(std::move(f));
        return cudaSuccess;
    }

    // Admit one request: assets resident and pinned, a framebuffer taken. Returns
    // AXR_E_BUDGET when it does not fit now (nothing changed), AXR_OK when admitted.
    axr_status admit(Req& q, bool* uploaded) {
        MeshAsset& m = *meshes[(size_t)q.r.mesh];
        Fb* fb = nullptr;
        for (auto& f : fbs)
            if (!f->busy && f->fb.width == q.r.width && f->fb.height == q.r.height) {
                fb = f.get();
                break;
            }
        uint64_t need = 0;
        if (!m.dev.pos) need += m.bytes();
        for (int32_t id : m.textures)
            if (!textures[(size_t)id]->dev.texels) need += textures[(size_t)id]->bytes();
        const size_t n = (size_t)q.r.width * (size_t)q.r.height;
        const size_t nt = (size_t)((q.r.width + kTile - 1) / kTile) * (size_t)((q.r.height + kTile - 1) / kTile);
        if (!fb) need += n * 16 + nt * 4;
        // pin what this request uses before evicting, so that eviction cannot take it
        ++m.pins;
        for (int32_t id : m.textures) ++textures[(size_t)id]->pins;
        if (fb) fb->busy = true;
        if (!make_room(need)) {
            --m.pins;
            for (int32_t id : m.textures) --textures[(size_t)id]->pins;
            if (fb) fb->busy = false;
            return AXR_E_BUDGET;
        }
        cudaError_t e = cudaSuccess;
        for (int32_t id : m.textures) {
            TexAsset& t = *textures[(size_t)id];
            if (!t.dev.texels && e == cudaSuccess) {
                e = upload_texture(t);
                *uploaded = true;
            }
            t.last_use = ++tick;
        }
        if (e == cudaSuccess && !m.dev.pos) {
            e = upload_mesh(m);
            *uploaded = true;
        } else if (e == cudaSuccess && m.mat_gen != tex_gen) {
            e = upload_materials(m);
            *uploaded = true;
        }
        if (e == cudaSuccess && !fb) e = new_framebuffer(q.r.width, q.r.height, &fb);
        if (e != cudaSuccess) {
            error = std::string("admission: ") + cudaGetErrorString(e);
            --m.pins;
            for (int32_t id : m.textures) --textures[(size_t)id]->pins;
            if (fb) fb->busy = false;
            return AXR_E_CUDA;
        }
        m.last_use = ++tick;
        fb->busy = true;
        fb->last_use = ++tick;
        q.fb = fb;
        return AXR_OK;
    }

    void release(Req& q) {
        MeshAsset& m = *meshes[(size_t)q.r.mesh];
        --m.pins;
        for (int32_t id : m.textures) --textures[(size_t)id]->pins;
        if (q.fb) {
            q.fb->busy = false;
            q.fb->last_use = ++tick;
            q.fb = nullptr;
        }
    }

    // ---------------------------------------------------------------- batches
    axr_status launch(Slot& s) {
    NvtxRange nvtx_range("axr_server batch");
        const uint64_t t = steady_ns();
        for (Req* q : s.reqs) q->launch = t;
        cudaError_t e = cudaSuccess;
        axr_context* ctx = s.sctx ? s.sctx : this->ctx;  // the stream and scratch the slot renders on
        if (cfg.per_request) {
            // the per-draw path for each request: clears, then drawMesh (tiled_pipeline.cpp:143)
            for (Req* q : s.reqs) {
                axr_framebuffer* fb = &q->fb->fb;
                const axr_server_request& r = q->r;
                axr_status st = AXR_OK;
                if (r.clear_flags & AXR_DRAW_CLEAR_COLOR)
                    st = axr_framebuffer_clear_color(ctx, fb, r.clear_rgba[0], r.clear_rgba[1], r.clear_rgba[2],
                                                     r.clear_rgba[3]);
                if (st == AXR_OK && (r.clear_flags & AXR_DRAW_CLEAR_DEPTH))
                    st = axr_framebuffer_clear_depth(ctx, fb, r.clear_depth);
                if (st == AXR_OK) st = axr_set_camera(ctx, &r.camera);
                if (st == AXR_OK) st = axr_set_shader(ctx, &r.shader);
                if (st == AXR_OK) st = axr_set_framebuffer(ctx, fb);
                if (st == AXR_OK) st = axr_draw_mesh(ctx, &meshes[(size_t)r.mesh]->dev, r.model);
                if (st != AXR_OK) return st;
            }
        } else {
            std::vector<axr_draw_desc> d(s.reqs.size());
            for (size_t k = 0; k < s.reqs.size(); ++k) {
                const axr_server_request& r = s.reqs[k]->r;
                axr_draw_desc& x = d[k];
                x.mesh = &meshes[(size_t)r.mesh]->dev;
                x.framebuffer = &s.reqs[k]->fb->fb;
                std::memcpy(x.model, r.model, sizeof(x.model));
                x.camera = r.camera;
                x.shader = r.shader;
                x.clear_flags = r.clear_flags;
                std::memcpy(x.clear_rgba, r.clear_rgba, 4);
                x.clear_depth = r.clear_depth;
            }
            std::lock_guard<std::mutex> lk(ctx->mu);
            axr_status st = batch_plan(ctx, d.data(), (int32_t)d.size(), &s.plan, true);
            if (st != AXR_OK) return st;
            if ((st = batch_launch(ctx, &s.plan)) != AXR_OK) return st;
        }
        // PNG files of the requests that ask for them, encoded behind the kernels
        s.files_pending = false;
        s.files_issued = false;
        for (int c = 0; c < 2; ++c) {
            s.png_reqs[c].clear();
            for (Req* q : s.reqs)
                if (q->r.png_channels == (uint32_t)(3 + c)) s.png_reqs[c].push_back(q);
            if (s.png_reqs[c].empty()) continue;
            axr_status st = s.png[c] ? AXR_OK : png_batch_create(ctx, &s.png[c]);
            std::vector<const axr_framebuffer*> f;
            for (Req* q : s.png_reqs[c]) f.push_back(&q->fb->fb);
            if (st == AXR_OK) {
                std::lock_guard<std::mutex> lk(ctx->mu);
                st = png_batch_encode_locked(ctx, s.png[c], (int32_t)f.size(), f.data(), (uint32_t)(3 + c));
            }
            if (st != AXR_OK) return st;
            s.files_pending = true;
        }
        // read-backs on the copy stream, behind the kernels
        e = cudaEventRecord(s.kernel_done, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(copy, s.kernel_done, 0);
        for (Req* q : s.reqs) {
            const size_t n = (size_t)q->r.width * (size_t)q->r.height;
            if (e == cudaSuccess && q->r.out_bgra)
                e = cudaMemcpyAsync(q->r.out_bgra, q->fb->fb.color, n * 4, cudaMemcpyDeviceToHost, copy);
            if (e == cudaSuccess && q->r.out_depth)
                e = cudaMemcpyAsync(q->r.out_depth, q->fb->fb.depth, n * 4, cudaMemcpyDeviceToHost, copy);
        }
        if (e == cudaSuccess) e = cudaEventRecord(s.copies_done, copy);
        if (e != cudaSuccess) {
            error = std::string("launch: ") + cudaGetErrorString(e);
            return AXR_E_CUDA;
        }
        ++stats.batches;
        return AXR_OK;
    }

    void finish(Req& q, int status) {
        q.status = status != AXR_OK ? status : q.png_status;
        q.done = steady_ns();
        q.finished = true;
        release(q);
        ++stats.completed;
    }

    // Issue the copies of a slot's PNG files once their encode is done; false while not.
    bool issue_files(Slot& s) {
        for (int c = 0; c < 2; ++c)
            if (!s.png_reqs[c].empty() && png_batch_query(s.png[c]) == cudaErrorNotReady) return false;
        cudaError_t e = cudaSuccess;
        for (int c = 0; c < 2; ++c) {
            for (size_t i = 0; i < s.png_reqs[c].size(); ++i) {
                Req* q = s.png_reqs[c][i];
                const void* dev = nullptr;
                uint64_t size = 0;
                png_batch_file(s.png[c], (int32_t)i, &dev, &size);
                q->png_bytes = size;
                if (size == 0) {
                    q->png_status = AXR_E_CUDA;
                } else if (size > q->r.out_png_capacity) {
                    q->png_status = AXR_E_CAPACITY;
                } else if (e == cudaSuccess) {
                    e = cudaMemcpyAsync(q->r.out_png, dev, size, cudaMemcpyDeviceToHost, copy);
                }
            }
        }
        if (e == cudaSuccess) e = cudaEventRecord(s.files_done, copy);
        if (e != cudaSuccess) {
            error = std::string("PNG read-back: ") + cudaGetErrorString(e);
            for (int c = 0; c < 2; ++c)
                for (Req* q : s.png_reqs[c]) q->png_status = AXR_E_CUDA;
        }
        s.files_issued = true;
        return true;
    }

    // Retire the busy slots whose read-backs are done (in launch order).
    bool retire() {
        bool any = false;
        for (auto& sp : slots) {
            Slot& s = *sp;
            if (!s.busy) continue;
            if (s.files_pending && !s.files_issued && !issue_files(s)) continue;
            cudaError_t e = cudaEventQuery(s.files_pending ? s.files_done : s.copies_done);
            if (e == cudaErrorNotReady) continue;
            const int status = e == cudaSuccess ? AXR_OK : AXR_E_CUDA;
            if (e != cudaSuccess) error = std::string("batch: ") + cudaGetErrorString(e);
            for (Req* q : s.reqs) finish(*q, status);
            s.reqs.clear();
            s.busy = false;
            any = true;
        }
        return any;
    }

    void run() {
        cudaSetDevice(cfg.device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            if (retire()) cv_done.notify_all();
            Slot* free_slot = nullptr;
            bool busy = false;
            for (auto& s : slots) {
                if (!s->busy && !free_slot) free_slot = s.get();
                busy |= s->busy;
            }
            if (stop && pending.empty() && !busy) break;
            if (free_slot && !pending.empty() && (!hold || stop)) {
                bool did_upload = false;
                while (!pending.empty() && (int32_t)free_slot->reqs.size() < cfg.max_batch) {
                    Req* q = pending.front();
                    const axr_status st = admit(*q, &did_upload);
                    if (st == AXR_E_BUDGET) {
                        if (free_slot->reqs.empty() && !busy) {  // cannot fit even with nothing in flight
                            pending.pop_front();
                            q->status = AXR_E_BUDGET;
                            q->done = steady_ns();
                            q->finished = true;
                            ++stats.completed;
                            cv_done.notify_all();
                            continue;
                        }
                        break;
                    }
                    pending.pop_front();
                    if (st != AXR_OK) {
                        q->status = st;
                        q->done = steady_ns();
                        q->finished = true;
                        ++stats.completed;
                        cv_done.notify_all();
                        continue;
                    }
                    free_slot->reqs.push_back(q);
                }
                if (!free_slot->reqs.empty()) {
                    // the slot's stream waits for the uploads and, when it is not the home
                    // stream, for the home stream's framebuffer allocations and frees
                    cudaStream_t ss = free_slot->sctx ? free_slot->sctx->stream : ctx->stream;
                    cudaError_t e = cudaSuccess;
                    if (ss != ctx->stream) {
                        e = cudaEventRecord(home_ready, ctx->stream);
                        if (e == cudaSuccess) e = cudaStreamWaitEvent(ss, home_ready, 0);
                    }
                    if (e == cudaSuccess && did_upload) {
                        e = cudaEventRecord(uploaded, upload);
                        if (e == cudaSuccess) e = cudaStreamWaitEvent(ss, uploaded, 0);
                    }
                    free_slot->id = next_batch++;
                    for (Req* q : free_slot->reqs) {
                        q->batch_id = free_slot->id;
                        q->batch_size = (uint32_t)free_slot->reqs.size();
                    }
                    const axr_status st = e == cudaSuccess ? launch(*free_slot) : AXR_E_CUDA;
                    if (st != AXR_OK) {
                        for (Req* q : free_slot->reqs) finish(*q, st);
                        free_slot->reqs.clear();
                        cv_done.notify_all();
                    } else {
                        free_slot->busy = true;
                    }
                    continue;
                }
            }
            // nothing to launch: wait for a request or a completion (polled)
            cv_work.wait_for(lk, std::chrono::microseconds(busy ? 20 : 1000));
        }
    }
};

extern "C" {

uint64_t axr_server_now_ns(void) { return steady_ns(); }

axr_status axr_server_create(const axr_server_config* cfg, axr_server** out) {
    if (!cfg || !out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    *out = nullptr;
    if (cfg->max_batch < 1 || cfg->max_inflight < 1 || cfg->memory_budget_bytes == 0)
        return fail(nullptr, AXR_E_INVALID, "server: max_batch, max_inflight and the budget must be positive");
    auto srv = std::make_unique<axr_server>();
    srv->cfg = *cfg;
    axr_status st = axr_context_create(cfg->device, &srv->ctx);
    if (st != AXR_OK) return st;
    DeviceGuard g(cfg->device);
    cudaError_t e = cudaStreamCreateWithFlags(&srv->upload, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&srv->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&srv->uploaded, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&srv->home_ready, cudaEventDisableTiming);
    for (int32_t k = 0; k < cfg->max_inflight && e == cudaSuccess; ++k) {
        auto s = std::make_unique<Slot>();
        st = cfg->overlap_kernels ? axr_context_create(cfg->device, &s->sctx) : AXR_OK;
        if (st != AXR_OK) {
            srv->slots.push_back(std::move(s));
            axr_server_destroy(srv.release());
            return st;
        }
        e = cudaEventCreateWithFlags(&s->kernel_done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->copies_done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->files_done, cudaEventDisableTiming);
        srv->slots.push_back(std::move(s));
    }
    if (e != cudaSuccess) {
        st = cuda_fail(nullptr, e, "server setup");
        axr_server_destroy(srv.release());
        return st;
    }
    axr_server* raw = srv.release();
    raw->worker = std::thread([raw] { raw->run(); });
    *out = raw;
    return AXR_OK;
}

void axr_server_destroy(axr_server* srv) {
    if (!srv) return;
    if (srv->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->stop = true;
        }
        srv->cv_work.notify_all();
        srv->worker.join();
    }
    if (srv->ctx) {
        DeviceGuard g(srv->cfg.device);
        cudaStreamSynchronize(srv->ctx->stream);
        if (srv->copy) cudaStreamSynchronize(srv->copy);
        if (srv->upload) cudaStreamSynchronize(srv->upload);
        for (auto& m : srv->meshes)
            if (m->dev.pos) srv->free_mesh_arrays(m->dev);
        for (auto& t : srv->textures)
            if (t->dev.texels) cudaFreeAsync(const_cast<uint32_t*>(t->dev.texels), srv->ctx->stream);
        for (auto& f : srv->fbs) srv->free_fb(*f);
        for (auto& s : srv->slots) {
            if (s->sctx) cudaStreamSynchronize(s->sctx->stream);
            free_batch(&s->plan);
            free_batch_staging(&s->plan);
            if (s->kernel_done) cudaEventDestroy(s->kernel_done);
            if (s->copies_done) cudaEventDestroy(s->copies_done);
            if (s->files_done) cudaEventDestroy(s->files_done);
            for (axr_png_batch* b : s->png) png_batch_release(b);
            if (s->sctx) axr_context_destroy(s->sctx);
        }
        cudaStreamSynchronize(srv->ctx->stream);
        if (srv->uploaded) cudaEventDestroy(srv->uploaded);
        if (srv->home_ready) cudaEventDestroy(srv->home_ready);
        if (srv->copy) cudaStreamDestroy(srv->copy);
        if (srv->upload) cudaStreamDestroy(srv->upload);
        axr_context_destroy(srv->ctx);
    }
    delete srv;
}

const char* axr_server_last_error(axr_server* srv) { return srv ? srv->error.c_str() : ""; }

axr_status axr_server_add_texture(axr_server* srv, const uint8_t* rgba, int32_t width, int32_t height, int32_t* out_id) {
    if (!srv || !rgba || !out_id || width <= 0 || height <= 0) return fail(nullptr, AXR_E_INVALID, "bad texture");
    auto t = std::make_unique<TexAsset>();
    t->width = width;
    t->height = height;
    if (!t->rgba.assign(rgba, (size_t)width * (size_t)height * 4)) return fail(nullptr, AXR_E_OOM, "pinned host memory");
    std::lock_guard<std::mutex> lk(srv->mu);
    *out_id = (int32_t)srv->textures.size();
    srv->textures.push_back(std::move(t));
    return AXR_OK;
}

axr_status axr_server_add_mesh(axr_server* srv, const axr_server_mesh_desc* d, int32_t* out_id) {
    if (!srv || !d || !out_id) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    if (d->num_vertices && (!d->positions || !d->uvs || !d->normals))
        return fail(nullptr, AXR_E_INVALID, "mesh needs positions, uvs and normals");
    if ((d->num_faces && !d->indices) || (d->num_groups && !d->groups) || (d->num_materials && !d->materials))
        return fail(nullptr, AXR_E_INVALID, "mesh arrays missing");
    auto m = std::make_unique<MeshAsset>();
    m->nv = d->num_vertices;
    m->nf = d->num_faces;
    for (uint64_t i = 0; i < 3ull * d->num_faces; ++i)
        if (d->indices[i] >= d->num_vertices) return fail(nullptr, AXR_E_INVALID, "face index out of range");
    std::lock_guard<std::mutex> lk(srv->mu);
    uint32_t base = 0;
    for (uint32_t k = 0; k < d->num_groups; ++k) {
        const axr_group_desc& g = d->groups[k];
        if ((uint64_t)g.start_face + g.face_count > d->num_faces || g.material >= d->num_materials)
            return fail(nullptr, AXR_E_INVALID, "group %u out of range", k);
        m->groups.push_back(DevGroup{g.start_face, g.face_count, base, g.material});
        base += g.face_count;
    }
    if (base > kMaxOrdinal + 1u) return fail(nullptr, AXR_E_CAPACITY, "a draw is limited to %u faces", kMaxOrdinal + 1u);
    m->num_drawn = base;
    for (uint32_t k = 0; k < d->num_materials; ++k) {
        const axr_server_material& sm = d->materials[k];
        for (int32_t id : {sm.diffuse, sm.bump, sm.metallic, sm.roughness, sm.ao}) {
            if (id >= (int32_t)srv->textures.size()) return fail(nullptr, AXR_E_INVALID, "material %u: texture %d", k, id);
            if (id >= 0 && std::find(m->textures.begin(), m->textures.end(), id) == m->textures.end())
                m->textures.push_back(id);
        }
        m->mats.push_back(sm);
    }
    auto widen = [&](HostBuf& dst, const float* src) {
        if (!src) return true;
        std::vector<float4> tmp(m->nv);
        for (uint32_t i = 0; i < m->nv; ++i) tmp[i] = make_float4(src[3ull * i], src[3ull * i + 1], src[3ull * i + 2], 0.f);
        return dst.assign(tmp.data(), sizeof(float4) * tmp.size());
    };
    bool ok = widen(m->pos, d->positions) && widen(m->nrm, d->normals) && widen(m->tan, d->tangents) &&
              widen(m->bit, d->bitangents) && m->uv.assign(d->uvs, 8ull * m->nv) &&
              m->idx.assign(d->indices, 12ull * m->nf);
    if (!ok) return fail(nullptr, AXR_E_OOM, "pinned host memory");
    mesh_bounds(d->positions, d->num_vertices, m->bound_center, &m->bound_radius);
    *out_id = (int32_t)srv->meshes.size();
    srv->meshes.push_back(std::move(m));
    return AXR_OK;
}

axr_status axr_server_submit(axr_server* srv, const axr_server_request* r, uint64_t* ticket) {
    if (!srv || !r || !ticket) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    if (r->width <= 0 || r->height <= 0 || r->width > 32768 || r->height > 32768)
        return fail(nullptr, AXR_E_INVALID, "request %dx%d", r->width, r->height);
    if (r->shader.kind < AXR_SHADER_FLAT || r->shader.kind > AXR_SHADER_GOURAUD)
        return fail(nullptr, AXR_E_INVALID, "unknown shader kind %d", r->shader.kind);
    if (r->png_channels != 0 && r->png_channels != 3 && r->png_channels != 4)
        return fail(nullptr, AXR_E_INVALID, "png_channels must be 0, 3 or 4");
    if (r->png_channels && !r->out_png) return fail(nullptr, AXR_E_INVALID, "a PNG request needs out_png");
    auto q = std::make_unique<Req>();
    q->r = *r;
    q->arrival = r->arrival_ns ? r->arrival_ns : steady_ns();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (r->mesh < 0 || r->mesh >= (int32_t)srv->meshes.size())
            return fail(nullptr, AXR_E_INVALID, "unknown mesh asset %d", r->mesh);
        *ticket = srv->next_ticket++;
        srv->pending.push_back(q.get());
        srv->reqs.emplace(*ticket, std::move(q));
        ++srv->stats.submitted;
    }
    srv->cv_work.notify_one();
    return AXR_OK;
}

axr_status axr_server_wait(axr_server* srv, uint64_t ticket, int32_t timeout_ms, axr_server_result* out) {
    if (!srv || !out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return fail(nullptr, AXR_E_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
    Req* q = it->second.get();
    auto done = [&] { return q->finished; };
    if (timeout_ms < 0)
        srv->cv_done.wait(lk, done);
    else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
        return AXR_E_TIMEOUT;
    out->status = q->status;
    out->batch_size = q->batch_size;
    out->arrival_ns = q->arrival;
    out->launch_ns = q->launch;
    out->done_ns = q->done;
    out->batch_id = q->batch_id;
    out->png_bytes = q->png_bytes;
    srv->reqs.erase(it);
    return AXR_OK;
}

axr_status axr_server_cancel(axr_server* srv, uint64_t ticket) {
    if (!srv) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        auto it = srv->reqs.find(ticket);
        if (it == srv->reqs.end()) return fail(nullptr, AXR_E_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
        Req* q = it->second.get();
        if (q->finished) return fail(nullptr, AXR_E_INVALID, "request %llu is done", (unsigned long long)ticket);
        auto pos = std::find(srv->pending.begin(), srv->pending.end(), q);
        if (pos == srv->pending.end())
            return fail(nullptr, AXR_E_INVALID, "request %llu is already in a batch", (unsigned long long)ticket);
        srv->pending.erase(pos);
        q->status = AXR_E_CANCELLED;
        q->done = steady_ns();
        q->finished = true;
        ++srv->stats.completed;
    }
    srv->cv_done.notify_all();
    return AXR_OK;
}

axr_status axr_server_hold(axr_server* srv, int32_t hold) {
    if (!srv) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->hold = hold != 0;
    }
    srv->cv_work.notify_all();
    return AXR_OK;
}

axr_status axr_server_get_stats(axr_server* srv, axr_server_stats* out) {
    if (!srv || !out) return fail(nullptr, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    *out = srv->stats;
    return AXR_OK;
}

}  // extern "C"
