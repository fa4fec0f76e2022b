/* Oracle test infrastructure: TiledPipeline::drawMesh restated in C (reference
 * src/tiled_pipeline.cpp:143-322), with the reference's stage structure:
 *   1. clip stage: faces of each material group split into contiguous per-thread chunks
 *      (cpp:181-190); per face the vertices are transformed by mvp (210-212), clipped
 *      (217 -> pipeline.cpp:176-228), culled (225) and set up (227-234); thread lists
 *      are appended in thread order, i.e. face order (250-259);
 *   2. initializeTiles + binTrianglesToTiles, serial (333-393), 16x16 tiles;
 *   3. tile workers pull batches of 8 non-empty tiles from an atomic counter (281-301);
 *      per tile and per triangle in bin order: vertex shader x3 (407-409) then the
 *      8-lane rasteriser with early depth test (rasterizeTriangleInTile_AVX256, 427-594);
 *   4. mergeTileResults, serial (1125-1181): strict less-than depth merge, RGBA -> BGRA.
 * The 8-lane AVX arithmetic is restated lane by lane; every lane operation is a single
 * IEEE float operation, so the results are identical.
 *
 * Differences that do not change the image, each stated where it occurs:
 *   - the 16 MiB triangle arena limit (tiled_pipeline.hpp:98-104) is not restated; the
 *     port draws any number of triangles in one pass;
 *   - triangles of earlier material groups are not re-appended for later groups
 *     (cpp:174/192/251-258 never clear threadClipped); the re-appended copies come later
 *     in bin order with the same depth, so a strict less-than test never lets them win;
 *   - each triangle is shaded with its own group's material (cpp:405 writes the shared
 *     shader's material from every worker, a race with more than one group);
 *   - the merge compares pixel by pixel instead of 8-wide blocks that may run past the
 *     tile's right edge when the framebuffer width is not a multiple of 8 (cpp:1145-1156). */
#include <pthread.h>
#include <stdint.h>
#include <unistd.h>
#include <stdlib.h>
#include <string.h>

#include "axo_port.h"

/* ------------------------------------------------------------------ thread pool */
typedef void (*task_fn)(void* arg, int tid, int nthreads);

#define POOL_MAX 256
static struct {
    pthread_t th[POOL_MAX];
    int nworkers;
    pthread_mutex_t mu;
    pthread_cond_t start, done;
    unsigned gen;
    int active, pending;
    task_fn fn;
    void* arg;
} g_pool = {.mu = PTHREAD_MUTEX_INITIALIZER, .start = PTHREAD_COND_INITIALIZER, .done = PTHREAD_COND_INITIALIZER};
static pthread_mutex_t g_render_mu = PTHREAD_MUTEX_INITIALIZER;

static void* pool_worker(void* p) {
    int tid = (int)(intptr_t)p;
    unsigned seen = 0;
    pthread_mutex_lock(&g_pool.mu);
    for (;;) {
        while (g_pool.gen == seen) pthread_cond_wait(&g_pool.start, &g_pool.mu);
        seen = g_pool.gen;
        if (tid < g_pool.active) {
            task_fn fn = g_pool.fn;
            void* arg = g_pool.arg;
            int n = g_pool.active;
            pthread_mutex_unlock(&g_pool.mu);
            fn(arg, tid, n);
            pthread_mutex_lock(&g_pool.mu);
            if (--g_pool.pending == 0) pthread_cond_signal(&g_pool.done);
        }
    }
    return NULL;
}

/* Runs fn(arg, tid, n) for tid = 0..n-1; the caller's thread is tid 0. */
static void parallel_run(int n, task_fn fn, void* arg) {
    if (n <= 1) { fn(arg, 0, 1); return; }
    if (n > POOL_MAX) n = POOL_MAX;
    pthread_mutex_lock(&g_pool.mu);
    while (g_pool.nworkers < n - 1) {
        int tid = g_pool.nworkers + 1;
        pthread_create(&g_pool.th[g_pool.nworkers], NULL, pool_worker, (void*)(intptr_t)tid);
        pthread_detach(g_pool.th[g_pool.nworkers]);
        g_pool.nworkers++;
    }
    g_pool.fn = fn;
    g_pool.arg = arg;
    g_pool.active = n;
    g_pool.pending = n - 1;
    g_pool.gen++;
    pthread_cond_broadcast(&g_pool.start);
    pthread_mutex_unlock(&g_pool.mu);
    fn(arg, 0, n);
    pthread_mutex_lock(&g_pool.mu);
    while (g_pool.pending > 0) pthread_cond_wait(&g_pool.done, &g_pool.mu);
    pthread_mutex_unlock(&g_pool.mu);
}

static int hw_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

/* ------------------------------------------------------------------ records */
typedef struct {
    float s[6];     /* screenPos x0,y0,x1,y1,x2,y2 */
    float z[3];     /* ndcZ */
    float minx, miny, maxx, maxy;
    cvert v[3];     /* Triangle::vertices (the Vertex part of each ClippedVertex) */
    uint32_t material;
} tri_t;

typedef struct {
    tri_t* data;
    size_t n, cap;
} tri_vec;

static void tri_push(tri_vec* v, const tri_t* t) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 1024;
        v->data = (tri_t*)realloc(v->data, v->cap * sizeof(tri_t));
    }
    v->data[v->n++] = *t;
}

typedef struct {
    uint32_t* idx;
    uint32_t n, cap;
} bin_t;

static void bin_push(bin_t* b, uint32_t t) {
    if (b->n == b->cap) {
        b->cap = b->cap ? b->cap * 2 : 16;
        b->idx = (uint32_t*)realloc(b->idx, b->cap * sizeof(uint32_t));
    }
    b->idx[b->n++] = t;
}

/* ------------------------------------------------------------------ clip stage */
typedef struct {
    const axo_mesh* mesh;
    const shader_state* sh;
    int width, height;
    uint32_t start, count, material;
    tri_vec* out; /* one per thread */
} clip_job;

static v3 vec3_at(const float* a, uint32_t i) { return a ? V3(a[3 * i], a[3 * i + 1], a[3 * i + 2]) : V3(0, 0, 0); }

static void clip_task(void* p, int tid, int nthreads) {
    clip_job* j = (clip_job*)p;
    const axo_mesh* m = j->mesh;
    int fpt = (int)((j->count + (uint32_t)nthreads - 1) / (uint32_t)nthreads);
    int start = (int)j->start + tid * fpt;
    int end = start + fpt;
    if (end > (int)(j->start + j->count)) end = (int)(j->start + j->count);
    cvert cv[MAX_CLIPPED_VERTS];
    for (int f = start; f < end; ++f) {
        for (int k = 0; k < 3; ++k) {
            uint32_t vi = m->indices[3 * (size_t)f + k];
            cvert* c = &cv[k];
            c->pos = vec3_at(m->positions, vi);
            c->uv = V2(m->uvs[2 * (size_t)vi], m->uvs[2 * (size_t)vi + 1]);
            c->nrm = vec3_at(m->normals, vi);
            c->tan = vec3_at(m->tangents, vi);
            c->bit = vec3_at(m->bitangents, vi);
            c->clip = m4v(&j->sh->mvp, V4(c->pos.x, c->pos.y, c->pos.z, 1.0f));
        }
        int n = port_clip(cv, 3);
        for (int q = 0; q + 2 < n; q += 3) {
            if (port_backface(&cv[q], &cv[q + 1], &cv[q + 2], j->width, j->height)) continue;
            tri_t t;
            float o[13];
            port_setup(&cv[q], j->width, j->height, o);
            memcpy(t.s, o, 6 * sizeof(float));
            memcpy(t.z, o + 6, 3 * sizeof(float));
            t.minx = o[9]; t.miny = o[10]; t.maxx = o[11]; t.maxy = o[12];
            t.v[0] = cv[q]; t.v[1] = cv[q + 1]; t.v[2] = cv[q + 2];
            t.material = j->material;
            tri_push(&j->out[tid], &t);
        }
    }
}

/* ------------------------------------------------------------------ raster stage */
typedef struct {
    int startx, starty, endx, endy;
} tile_rect;

typedef struct {
    const tri_t* tris;
    const bin_t* bins;
    const uint32_t* relevant; /* tile indices with a non-empty bin, ascending */
    uint32_t nrel;
    const tile_rect* tiles;
    const shader_state* sh;
    const axo_mesh* mesh;
    uint8_t* res_color; /* nrel * 16*16*4 */
    float* res_depth;   /* nrel * 16*16 */
    int next_batch;     /* atomic */
} raster_job;

static uint8_t quantize(float c) { return (uint8_t)(clampf_std(c, 0.0f, 1.0f) * 255.0f); }

/* rasterizeTriangleInTile_AVX256, tiled_pipeline.cpp:427-594 */
static void raster_tri(const tri_t* tri, const tile_rect* tile, const shader_state* sh, const axo_material* mat,
                       const vsout vs[3], uint8_t* color, float* depth) {
    int bx0 = (int)floorf(tri->minx), by0 = (int)floorf(tri->miny);
    int bx1 = (int)ceilf(tri->maxx), by1 = (int)ceilf(tri->maxy);
    int startx = tile->startx > bx0 ? tile->startx : bx0;
    int starty = tile->starty > by0 ? tile->starty : by0;
    int endx = tile->endx < bx1 ? tile->endx : bx1;
    int endy = tile->endy < by1 ? tile->endy : by1;
    if (startx >= endx || starty >= endy) return;
    float x0 = tri->s[0], y0 = tri->s[1], x1 = tri->s[2], y1 = tri->s[3], x2 = tri->s[4], y2 = tri->s[5];
    float e0c = x1 * y2 - x2 * y1;
    float e1c = x2 * y0 - x0 * y2;
    float e2c = x0 * y1 - x1 * y0;
    float area = e0c + e1c + e2c;
    if (area >= 0 && (double)area < 1.0E-12) return;
    float e0a = y1 - y2, e0b = x2 - x1;
    float e1a = y2 - y0, e1b = x0 - x2;
    float e2a = y0 - y1, e2b = x1 - x0;
    if (area < 0) {
        e0a = -e0a; e0b = -e0b; e0c = -e0c;
        e1a = -e1a; e1b = -e1b; e1c = -e1c;
        e2a = -e2a; e2b = -e2b; e2c = -e2c;
        area = -area;
    }
    float inv_area = 1.0f / area;
    for (int py = starty; py < endy; ++py) {
        float pyc = (float)py + 0.5f;
        float r0 = e0a * ((float)startx + 0.5f) + e0b * pyc + e0c;
        float r1 = e1a * ((float)startx + 0.5f) + e1b * pyc + e1c;
        float r2 = e2a * ((float)startx + 0.5f) + e2b * pyc + e2c;
        for (int px = startx; px < endx; px += 8) {
            float c0[8], c1[8], c2[8];
            int mask = 0;
            for (int i = 0; i < 8; ++i) {
                c0[i] = r0 + e0a * (float)i;
                c1[i] = r1 + e1a * (float)i;
                c2[i] = r2 + e2a * (float)i;
                if (c0[i] >= 0.f && c1[i] >= 0.f && c2[i] >= 0.f) mask |= 1 << i;
            }
            if (mask) {
                for (int i = 0; i < 8; ++i) {
                    if (!(mask & (1 << i))) continue;
                    int cx = px + i;
                    if (cx >= endx) break;
                    float alpha = c0[i] * inv_area;
                    float beta = c1[i] * inv_area;
                    float gamma = c2[i] * inv_area;
                    float z = tri->z[0] * alpha + tri->z[1] * beta + tri->z[2] * gamma;
                    int idx = (py - tile->starty) * TILE_SIZE + (cx - tile->startx);
                    if (z < depth[idx]) {
                        v4 c = shader_fragment(sh, mat, V3(alpha, beta, gamma), vs);
                        depth[idx] = z;
                        color[4 * idx + 0] = quantize(c.x);
                        color[4 * idx + 1] = quantize(c.y);
                        color[4 * idx + 2] = quantize(c.z);
                        color[4 * idx + 3] = quantize(c.w);
                    }
                }
            }
            r0 += e0a * 8.0f;
            r1 += e1a * 8.0f;
            r2 += e2a * 8.0f;
        }
    }
}

static void raster_task(void* p, int tid, int nthreads) {
    raster_job* j = (raster_job*)p;
    uint8_t color[TILE_SIZE * TILE_SIZE * 4];
    float depth[TILE_SIZE * TILE_SIZE];
    uint32_t nbatches = (j->nrel + BATCH_SIZE - 1) / BATCH_SIZE;
    for (;;) {
        uint32_t b = (uint32_t)__atomic_fetch_add(&j->next_batch, 1, __ATOMIC_RELAXED);
        if (b >= nbatches) break;
        uint32_t e = (b + 1) * BATCH_SIZE < j->nrel ? (b + 1) * BATCH_SIZE : j->nrel;
        for (uint32_t r = b * BATCH_SIZE; r < e; ++r) {
            uint32_t ti = j->relevant[r];
            const tile_rect* tile = &j->tiles[ti];
            memset(color, 0, sizeof(color));
            for (int k = 0; k < TILE_SIZE * TILE_SIZE; ++k) depth[k] = INFINITY;
            const bin_t* bin = &j->bins[ti];
            for (uint32_t q = 0; q < bin->n; ++q) {
                const tri_t* tri = &j->tris[bin->idx[q]];
                vsout vs[3];
                for (int k = 0; k < 3; ++k) vs[k] = shader_vertex(j->sh, &tri->v[k]);
                raster_tri(tri, tile, j->sh, &j->mesh->materials[tri->material], vs, color, depth);
            }
            memcpy(j->res_color + (size_t)r * sizeof(color), color, sizeof(color));
            memcpy(j->res_depth + (size_t)r * TILE_SIZE * TILE_SIZE, depth, sizeof(depth));
        }
    }
}

/* ------------------------------------------------------------------ draw */
int port_draw(const axo_mesh* mesh, const float* model, const float* view_proj, const float* cam_pos,
              const axo_shader* shader, int width, int height, int threads, uint8_t* bgra, float* depth) {
    if (shader->kind < AXO_FLAT || shader->kind > AXO_GOURAUD || width <= 0 || height <= 0) return 1;
    for (uint32_t g = 0; g < mesh->num_groups; ++g) {
        const uint32_t* gr = mesh->groups + 3 * g;
        if ((uint64_t)gr[0] + gr[1] > mesh->num_faces || gr[2] >= mesh->num_materials) return 1;
    }
    pthread_mutex_lock(&g_render_mu);
    int nthreads = threads > 0 ? threads : hw_threads();
    m4 M = m4_load(model), vp = m4_load(view_proj);
    shader_state sh;
    shader_init(&sh, shader, &M, &vp, V3(cam_pos[0], cam_pos[1], cam_pos[2]));

    /* 1. clip stage, per material group (cpp:176-260) */
    tri_vec all = {0};
    tri_vec* per = (tri_vec*)calloc((size_t)nthreads, sizeof(tri_vec));
    for (uint32_t g = 0; g < mesh->num_groups; ++g) {
        clip_job job = {mesh, &sh, width, height, mesh->groups[3 * g], mesh->groups[3 * g + 1],
                        mesh->groups[3 * g + 2], per};
        for (int t = 0; t < nthreads; ++t) per[t].n = 0;
        parallel_run(nthreads, clip_task, &job);
        for (int t = 0; t < nthreads; ++t)
            for (size_t q = 0; q < per[t].n; ++q) tri_push(&all, &per[t].data[q]);
    }
    for (int t = 0; t < nthreads; ++t) free(per[t].data);
    free(per);

    /* 2. tiles and bins (cpp:333-393) */
    int ntx = (width + TILE_SIZE - 1) / TILE_SIZE;
    int nty = (height + TILE_SIZE - 1) / TILE_SIZE;
    size_t ntiles = (size_t)ntx * (size_t)nty;
    tile_rect* tiles = (tile_rect*)malloc(ntiles * sizeof(tile_rect));
    bin_t* bins = (bin_t*)calloc(ntiles, sizeof(bin_t));
    for (int ty = 0; ty < nty; ++ty)
        for (int tx = 0; tx < ntx; ++tx) {
            tile_rect* t = &tiles[(size_t)ty * ntx + tx];
            t->startx = tx * TILE_SIZE;
            t->starty = ty * TILE_SIZE;
            t->endx = (tx + 1) * TILE_SIZE < width ? (tx + 1) * TILE_SIZE : width;
            t->endy = (ty + 1) * TILE_SIZE < height ? (ty + 1) * TILE_SIZE : height;
        }
    for (size_t q = 0; q < all.n; ++q) {
        const tri_t* tr = &all.data[q];
        int stx = (int)tr->minx / TILE_SIZE; if (stx < 0) stx = 0;
        int sty = (int)tr->miny / TILE_SIZE; if (sty < 0) sty = 0;
        int etx = (int)tr->maxx / TILE_SIZE; if (etx > ntx - 1) etx = ntx - 1;
        int ety = (int)tr->maxy / TILE_SIZE; if (ety > nty - 1) ety = nty - 1;
        for (int ty = sty; ty <= ety; ++ty)
            for (int tx = stx; tx <= etx; ++tx) {
                size_t ti = (size_t)ty * ntx + tx;
                const tile_rect* t = &tiles[ti];
                /* triangleIntersectsTile, cpp:356-366 */
                if (tr->maxx < (float)t->startx || tr->minx > (float)t->endx || tr->maxy < (float)t->starty ||
                    tr->miny > (float)t->endy)
                    continue;
                bin_push(&bins[ti], (uint32_t)q);
            }
    }
    /* preprocessTiles, cpp:324-331 */
    uint32_t* relevant = (uint32_t*)malloc(ntiles * sizeof(uint32_t));
    uint32_t nrel = 0;
    for (size_t ti = 0; ti < ntiles; ++ti)
        if (bins[ti].n) relevant[nrel++] = (uint32_t)ti;

    /* 3. tile workers (cpp:281-309) */
    raster_job rj = {all.data, bins, relevant, nrel, tiles, &sh, mesh,
                     (uint8_t*)malloc((size_t)nrel * TILE_SIZE * TILE_SIZE * 4 + 1),
                     (float*)malloc((size_t)nrel * TILE_SIZE * TILE_SIZE * sizeof(float) + 1), 0};
    parallel_run(nthreads, raster_task, &rj);

    /* 4. mergeTileResults (cpp:1125-1181) */
    for (uint32_t r = 0; r < nrel; ++r) {
        const tile_rect* t = &tiles[relevant[r]];
        const uint8_t* tc = rj.res_color + (size_t)r * TILE_SIZE * TILE_SIZE * 4;
        const float* tz = rj.res_depth + (size_t)r * TILE_SIZE * TILE_SIZE;
        for (int y = 0; y < t->endy - t->starty; ++y) {
            size_t row = (size_t)(t->starty + y) * (size_t)width + (size_t)t->startx;
            for (int x = 0; x < t->endx - t->startx; ++x) {
                int li = y * TILE_SIZE + x;
                if (tz[li] < depth[row + x]) {
                    depth[row + x] = tz[li];
                    uint8_t* o = bgra + 4 * (row + x);
                    o[0] = tc[4 * li + 2];
                    o[1] = tc[4 * li + 1];
                    o[2] = tc[4 * li + 0];
                    o[3] = tc[4 * li + 3];
                }
            }
        }
    }

    free(rj.res_color);
    free(rj.res_depth);
    free(relevant);
    for (size_t ti = 0; ti < ntiles; ++ti) free(bins[ti].idx);
    free(bins);
    free(tiles);
    free(all.data);
    pthread_mutex_unlock(&g_render_mu);
    return 0;
}

/* Camera(position, target, fov, aspect) + update(0), then port_draw with its matrices. */
int port_render(const axo_mesh* mesh, const float* model, const axo_camera* camera, const axo_shader* shader,
                int width, int height, int threads, int max_faces_per_draw, uint8_t* bgra, float* depth,
                float* matrices_out48) {
    (void)max_faces_per_draw; /* the port has no triangle arena limit */
    m4 view, proj, vp;
    port_camera_matrices(camera, &view, &proj, &vp);
    float m[48];
    m4_store(&view, m);
    m4_store(&proj, m + 16);
    m4_store(&vp, m + 32);
    if (matrices_out48) memcpy(matrices_out48, m, sizeof(m));
    return port_draw(mesh, model, m + 32, camera->position, shader, width, height, threads, bgra, depth);
}
